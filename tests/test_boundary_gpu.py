"""The compiled boundary on the GPU: the standalone C++ driver and the MEX
gateways (built against the project's mx stub) reproduce, through the C
ABI, what the oracle and the Python mirror give on the same inputs - the
sampler chain bit for bit, findROI's maxima, boxes, crops and flag image bit
for bit, gaussMLE's fits equal to the library's and within 1e-4 of the
oracle."""
import ctypes as C
import json
import struct

import numpy as np
import pytest

from bamf_gb300 import abi, rjstruct, sampler, synth
from mex_harness import Gateway, run_driver

pytestmark = pytest.mark.gpu


def _c0(steps=600, seed=0):
    b = synth.roi_batch_c0(4, seed=seed)
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = steps
    return b, rj, rjstruct.mcmc_params(rj), rjstruct.initial_bg(rj)


def _write_input(path, roi, p, rj, e0, rng, arith):
    ys, xs = roi.shape
    I, X, Y, BG = e0
    with open(path, "wb") as f:
        f.write(b"BAMFRJ1\0")
        f.write(struct.pack("<ii", xs, ys))
        f.write(bytes(p))
        f.write(struct.pack("<if", len(I), BG))
        for v in (I, X, Y):
            f.write(np.asarray(v, np.float32).tobytes())
        f.write(struct.pack("<IIIi", *rng, arith))
        for pdf in (rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons):
            a = np.asarray(pdf, np.float32)
            f.write(struct.pack("<i", a.size))
            f.write(a.tobytes())
        f.write(np.asarray(roi, np.float32).ravel(order="F").tobytes())


def _read_output(path, xs, ys, zoom):
    raw = open(path, "rb").read()
    assert raw[:8] == b"BAMFRO1\0"
    pos = 8
    st = struct.unpack_from("<i", raw, pos)[0]
    pos += 4
    assert st == 0, st
    out = {}

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(raw, dt, n, pos).copy()
        pos += a.nbytes
        return a

    for w in ("chain", "chain_test"):
        ne, nr = struct.unpack_from("<ii", raw, pos)
        pos += 8
        c = {}
        for name, dt in abi.ENTRY_FIELDS:
            c[name] = take(dt, ne)
        for name, dt in abi.RECORD_FIELDS:
            c[name] = take(dt, nr)
        out[w] = c
    G = struct.unpack_from("<q", raw, pos)[0]
    pos += 8
    out["pgrid"] = take(np.float32, G).reshape(xs * zoom, ys * zoom).T
    out["pback"] = take(np.float32, G).reshape(xs * zoom, ys * zoom).T
    cnt = take(np.int32, 30)
    out["counters"] = dict(zip(abi.COUNTER_NAMES, map(int, cnt)))
    return out


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float32:
        return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.astype(np.float32).view(np.uint32))
    return a.shape == b.shape and np.array_equal(a, b)


def test_driver_chain_matches_the_oracle_bit_for_bit(cuda_lib, oracle_port, tmp_path):
    """bamf_driver rjmcmc (C++ -> bamf_crjmcmc_host) on a ROI with a start
    state and a stream offset: every chain vector, the grids and the
    counters equal the oracle's."""
    b, rj, p, bg0 = _c0(steps=800, seed=2)
    k = 1
    e0 = (b.true_i[k].astype(np.float32), b.true_x[k].astype(np.float32), b.true_y[k].astype(np.float32), 9.0)
    rng = (17, 3, 40)
    _write_input(tmp_path / "in.bin", b.roi(k), p, rj, e0, rng, abi.BAMF_ARITH_EXACT)
    r = run_driver("rjmcmc", tmp_path / "in.bin", tmp_path / "out.bin")
    assert r.returncode == 0, r.stderr
    got = _read_output(tmp_path / "out.bin", 16, 16, int(p.Grid_Zoom))
    ref = oracle_port.run_chain("port", b.roi(k), p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, e0=e0,
                                rng=rng)
    for w in ("chain", "chain_test"):
        for f, v in ref[w].items():
            assert _same(got[w][f], v), (w, f)
    assert _same(got["pgrid"], ref["pgrid"]) and _same(got["pback"], ref["pback"])
    assert got["counters"] == ref["counters"]


def test_driver_batch_runs_the_uneven_workload(cuda_lib):
    """bamf_driver batch: 2000 generated uneven ROIs through
    bamf_rjmcmc_batch_host at the workload's 3000 + 3000 jumps; every ROI
    runs and the mean MAP count is near the generator's (the reference's
    moves overshoot in early burn-in, so short chains would not be)."""
    r = run_driver("batch", 2000, 3000, 7)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    print(line)
    assert line["roi_errors"] == 0 and line["rois_per_s"] > 0
    assert abs(line["map_n_mean"] - line["true_n_mean"]) < 0.5


def _mcmc_struct(p):
    return {"PSFsigma": float(p.PSFsigma), "N_Trials": float(p.N_Trials), "N_Burnin": float(p.N_Burnin),
            "I_stdFg": float(p.I_stdFg), "I_stdBg": float(p.I_stdBg), "X_stdFg": float(p.X_stdFg),
            "X_stdBg": float(p.X_stdBg), "P_Burnin": np.array(list(p.P_Burnin), np.float32),
            "P_Trials": np.array(list(p.P_Trials), np.float32), "Rho": float(p.Rho), "Bnd_out": float(p.Bnd_out),
            "Grid_Zoom": float(p.Grid_Zoom), "Split_std": float(p.Split_std), "Icutoff": float(p.Icutoff),
            "BG_std": float(p.BG_std), "ABBG_std": float(p.ABBG_std), "DX": float(p.DX), "DriftX": float(p.DriftX),
            "DriftY": float(p.DriftY), "PSFsize": np.array(list(p.PSFsize), np.int32), "IsBackg": float(p.IsBackg)}


def test_crjmcmc_gateway_marshals_the_reference_outputs(cuda_lib, oracle_port):
    """cRJMCMC_bamf called the way rjmcmc.m:102 calls cRJMCMC (single
    inputs, MCMC struct, zero sCMOS and sampled PSF, OptModel 0) plus the
    stream [seed chain offset]: PGrid / PBack are the oracle's; the
    accepted and proposed struct arrays hold the oracle chain as
    cRJMCMC.cpp:159-276 marshals it (the Python mirror sampler.mex_chain),
    with the last element empty; Stat is the 16 acceptance ratios."""
    b, rj, p, bg0 = _c0(steps=500, seed=4)
    k = 2
    roi = b.roi(k)
    ref = oracle_port.run_chain("port", roi, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons,
                                e0=([], [], [], bg0), rng=(5, 11, 0))
    g = Gateway("cRJMCMC_bamf")
    E = {"N": 0.0, "I": np.zeros(0, np.float32), "X": np.zeros(0, np.float32), "Y": np.zeros(0, np.float32),
         "BG": float(bg0)}
    pg, pb, chain, prop, stat = g(5, roi.astype(np.float32), E, _mcmc_struct(p), 16.0, 16.0,
                                  np.asarray(rj.P_Offset, np.float32), np.asarray(rj.P_EmPhotons, np.float32),
                                  np.asarray(rj.P_BgEmPhotons, np.float32), np.zeros((16, 16), np.float32),
                                  np.zeros((10, 10, 2, 2), np.float32), 0.0, "exact", np.array([5.0, 11.0]))
    assert _same(pg, ref["pgrid"]) and _same(pb, ref["pback"])
    want_a = sampler.mex_chain(ref["chain"])
    want_p = sampler.mex_chain(ref["chain_test"], accepted=ref["chain"])
    for got, want in ((chain, want_a), (prop, want_p)):
        assert len(got) == len(want) + 1 and all(v is None for v in got[-1].values())
        for gk, wk in zip(got[:-1], want):
            for f in ("N", "LLR", "PR", "JumpType", "Accepted", "BG", "ABG", "BBG"):
                assert float(np.asarray(gk[f]).ravel()[0]) == wk[f], f
            for f in ("X", "Y", "Photons", "Signal"):
                np.testing.assert_array_equal(np.asarray(gk[f]).ravel(), wk[f], err_msg=f)
    want_s = sampler.mex_stat(ref["counters"], p)
    for f, v in want_s.items():
        assert float(np.asarray(stat[f]).ravel()[0]) == pytest.approx(v, rel=1e-12), f


def test_findroi_gateway_matches_the_oracle(cuda_lib, oracle_port):
    stack, _ = synth.frames(6, size=96, seed=11)
    g = Gateway("findROI_bamf")
    smd, rois, res = g(3, stack.astype(np.float32), 1.3, 2.6, 7.0)
    ref = oracle_port.findroi(stack, 1.3, 2.6, 7)
    np.testing.assert_array_equal(np.asarray(smd["XBoxCorner"]).ravel(), ref["XBoxCorner"])
    np.testing.assert_array_equal(np.asarray(smd["YBoxCorner"]).ravel(), ref["YBoxCorner"])
    np.testing.assert_array_equal(np.asarray(smd["FrameNum"]).ravel(), ref["coords"][:, 2])
    assert rois.shape == ref["ROIStack"].shape and rois.dtype == np.float64
    np.testing.assert_array_equal(rois.astype(np.float32), ref["ROIStack"])
    np.testing.assert_array_equal(res.ravel(order="F"), ref["flags"].astype(np.float64))
    assert len(ref["XBoxCorner"]) > 50


@pytest.mark.parametrize("fit", ["Basic", "Sigma", "SigmaYX"])
def test_gaussmle_gateway_matches_the_library_and_the_oracle(cuda_lib, oracle_port, fit):
    from bamf_gb300 import frontend
    stack, _ = synth.frames(4, size=96, seed=12)
    rois = oracle_port.findroi(stack, 1.3, 2.6, 7)["ROIStack"].astype(np.float32)
    g = Gateway("gaussMLE_bamf")
    R, S = g(2, rois, fit, "CCD", 1.3, "Iterations", 10.0)
    lib = frontend.gaussMLE(rois, fit, "CCD", 1.3, Iterations=10)
    assert set(R) == set(lib)
    for f, v in lib.items():
        np.testing.assert_array_equal(np.asarray(R[f]).ravel(), np.asarray(v, np.float32), err_msg=f)
    assert S["NFitsPerCall"] == rois.shape[2]
    if fit == "Basic":
        ref = oracle_port.gaussmle(rois, 1.3, 10)
        P = np.stack([R["Y"].ravel(), R["X"].ravel(), R["Photons"].ravel(), R["BG"].ravel()], 1)
        rel = np.abs(P - ref["P"]) / np.maximum(np.abs(ref["P"]), 1e-3)
        assert np.percentile(rel, 99) < 1e-4
