"""Generates tests/golden/rjmcmc_ref_numpsf.npz from the reference sampler
with its sampled-PSF model (OptModel 1, NumModel in source/c/LibRJMCMC.cpp,
compiled unmodified by oracle/Makefile into oracle/_ref/).

Two cases, both on ROIs of synth.roi_batch_c0(seed=0) (16x16 px), the
settings of rjstruct.c0_rjstruct() with 1500 burn-in + 1500 trial jumps,
empty start (BG from the offset prior), uniform stream seed 11 with chain id
= ROI index:
  gauss64  40 ROIs, the pixel-integrated Gaussian PSF of sigma 1.3 sampled
           64 x 64 px at 4 x 4 sub-positions (psf.gaussian_sampled_psf);
  small10  10 ROIs, a 10 x 10 x 2 x 2 PSF (the shape rjmcmc.m passes by
           default) of uniform [0, 0.05) values, seed 1, whose flat indices
           leave the array for most emitter positions (reads clamped to the
           last element, one message each).
Stored per ROI and case: chain length, uniforms drawn, the 30 counters, the
message count and a SHA-256 of every output (Chain and Chain_Test vectors,
PGrid, PBack).

Usage (where the reference tree exists):  python tests/golden/make_numpsf_golden.py
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from bamf_gb300 import psf as psfmod, rjstruct, synth  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rjmcmc_ref_numpsf.npz")
SEED = 11
STEPS = 1500


def digest(res: dict) -> str:
    h = hashlib.sha256()
    for w in ("chain", "chain_test"):
        for k in sorted(res[w]):
            h.update(k.encode())
            h.update(np.ascontiguousarray(res[w][k]).tobytes())
    h.update(np.ascontiguousarray(res["pgrid"]).tobytes())
    h.update(np.ascontiguousarray(res["pback"]).tobytes())
    return h.hexdigest()


def cases():
    small = (np.random.default_rng(1).random((10, 10, 2, 2)) * 0.05).astype(np.float32)
    return {"gauss64": (psfmod.gaussian_sampled_psf(1.3), 40), "small10": (small, 10)}


def params(psf):
    rj = rjstruct.c0_rjstruct()
    rj.N_Burnin = rj.N_Trials = STEPS
    p = rjstruct.mcmc_params(rj)
    for k, v in enumerate(psf.shape):
        p.PSFsize[k] = v
    return rj, p


def main() -> None:
    oracle.build(ref=True)
    b = synth.roi_batch_c0(40, seed=0)
    out = {"seed": SEED, "steps": STEPS}
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for name, (psf, n) in cases().items():
            rj, p = params(psf)
            bg0 = rjstruct.initial_bg(rj)

            def one(k):
                r = oracle.run_chain("ref", b.roi(k), p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons,
                                     e0=([], [], [], bg0), rng=(SEED, k, 0), sampled_psf=psf)
                c = r["counters"]
                return (len(r["chain"]["N"]), r["uniforms_used"], [c[m] for m in sorted(c)], r["messages"],
                        digest(r))

            rows = list(ex.map(one, range(n)))
            out[f"{name}_entries"] = np.array([r[0] for r in rows], np.int64)
            out[f"{name}_uniforms"] = np.array([r[1] for r in rows], np.int64)
            out[f"{name}_counters"] = np.array([r[2] for r in rows], np.int64)
            out[f"{name}_messages"] = np.array([r[3] for r in rows], np.int64)
            out[f"{name}_sha256"] = np.array([r[4] for r in rows])
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
