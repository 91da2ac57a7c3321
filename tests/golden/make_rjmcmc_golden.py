"""Generates tests/golden/rjmcmc_ref_c0.npz from the reference sampler.

Runs the reference sampler (source/c/LibRJMCMC.cpp compiled unmodified by
oracle/Makefile into oracle/_ref/) on the plain-RJMCMC workload: 200 ROIs of
16x16 px from synth.roi_batch_c0(seed=0), 3000 burn-in + 3000 trial jumps,
the settings of rjstruct.c0_rjstruct(), empty start (BG from the offset
prior), uniform stream seed 7 with chain id = ROI index.

Stored per ROI, for both reference builds (parity math "pm" and glibc math
"native"): chain length, record count, uniforms drawn, the 30 counters and a
SHA-256 of every output (Chain and Chain_Test vectors, PGrid, PBack) so a
test can pin the CPU restatement to the reference without the reference
tree.  Also stored: the full raw outputs of three short runs (500 + 500),
and the fraction of ROIs whose accept/reject sequence is the same under
glibc math as under parity math.

Usage (where the reference tree exists):  python tests/golden/make_rjmcmc_golden.py
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
from bamf_gb300 import rjstruct, synth  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rjmcmc_ref_c0.npz")
SEED = 7
N_ROIS = 200


def digest(res: dict) -> str:
    h = hashlib.sha256()
    for w in ("chain", "chain_test"):
        for k in sorted(res[w]):
            h.update(k.encode())
            h.update(np.ascontiguousarray(res[w][k]).tobytes())
    h.update(np.ascontiguousarray(res["pgrid"]).tobytes())
    h.update(np.ascontiguousarray(res["pback"]).tobytes())
    return h.hexdigest()


def summary(res: dict):
    c = res["counters"]
    return (len(res["chain"]["N"]), len(res["chain"]["Index"]), res["uniforms_used"],
            [c[n] for n in sorted(c)], digest(res), res["chain"]["Accepted"].copy(),
            res["messages"])


def main() -> None:
    oracle.build(ref=True)
    b = synth.roi_batch_c0(N_ROIS, seed=0)
    rj = rjstruct.c0_rjstruct()
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    args = (p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons)

    def one(kind, k):
        return summary(oracle.run_chain(kind, b.roi(k), *args, e0=([], [], [], bg0), rng=(SEED, k, 0)))

    out = {"n_rois": N_ROIS, "seed": SEED, "counter_names": np.array(sorted(oracle_names()))}
    acc = {}
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for tag, kind in (("pm", "ref"), ("native", "ref_native")):
            rows = list(ex.map(lambda k: one(kind, k), range(N_ROIS)))
            out[f"{tag}_entries"] = np.array([r[0] for r in rows], np.int64)
            out[f"{tag}_records"] = np.array([r[1] for r in rows], np.int64)
            out[f"{tag}_uniforms"] = np.array([r[2] for r in rows], np.int64)
            out[f"{tag}_counters"] = np.array([r[3] for r in rows], np.int64)
            out[f"{tag}_sha256"] = np.array([r[4] for r in rows])
            out[f"{tag}_messages"] = np.array([r[6] for r in rows], np.int64)
            acc[tag] = [r[5] for r in rows]
    same = [a.shape == n.shape and np.array_equal(a, n) for a, n in zip(acc["pm"], acc["native"])]
    out["native_same_accept_fraction"] = float(np.mean(same))

    rj_s = rjstruct.c0_rjstruct()
    rj_s.N_Burnin = rj_s.N_Trials = 500
    ps = rjstruct.mcmc_params(rj_s)
    for k in range(3):
        res = oracle.run_chain("ref", b.roi(k), ps, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons,
                               e0=([], [], [], bg0), rng=(SEED, k, 0))
        for w in ("chain", "chain_test"):
            for f, v in res[w].items():
                out[f"short{k}_{w}_{f}"] = v
        out[f"short{k}_pgrid"] = res["pgrid"]
        out[f"short{k}_counters"] = np.array([res["counters"][n] for n in sorted(res["counters"])])
        out[f"short{k}_uniforms"] = res["uniforms_used"]
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: native math keeps the accept sequence on "
          f"{out['native_same_accept_fraction']*100:.1f}% of ROIs")


def oracle_names():
    from bamf_gb300.abi import COUNTER_NAMES
    return COUNTER_NAMES


if __name__ == "__main__":
    main()
