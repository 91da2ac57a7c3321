"""Learned vs uniform proposals on 16x16 ROIs: throughput, effective
samples per second, MAP emitter-count accuracy and localisation error.

Protocol (all on one GPU):
  1. train the proposal network on `train_rois` generator ROIs (Poisson(5)
     emitters, the plain-RJMCMC generator otherwise);
  2. draw `n_eval` fresh ROIs from the same generator (another seed);
  3. run the batched fast sampler with UNIFORM and with LEARNED proposals
     (birth, split and relocation from the network's density; its inference
     time counts against the learned arm), M = 4 chains per ROI from
     dispersed start states (0, 2, 8 and 12 emitters at uniform positions,
     the same for every arm; the learned_init arm starts its first chain
     from the network's state instead of the empty one), each chain
     recording its per-entry emitter-count and mean-X traces;
  4. per ROI of a subset, the rank-normalised split-R-hat and the
     multi-chain bulk ESS of both traces over the second half of the
     chains (bamf_gb300.ess, Vehtari et al. 2021); ESS per chain times the
     arm's chains per second is its ESS/s;
  5. MAP emitter-count accuracy and the localisation RMSE of the final
     state's emitters matched to the truth (Hungarian matching on ROIs
     whose final count equals the true count), from each ROI's first chain;
  6. equal accuracy: a sweep of chain lengths finds the shortest learned
     run whose MAP count accuracy reaches the uniform arm's full-length
     accuracy AND whose RMSE is within 5% of the uniform arm's; the
     throughput ratio at that length is reported with both figures.
"""
from __future__ import annotations

import time

import numpy as np

from . import ess, learned, rjstruct, sampler


def _rj(jumps: int):
    rj = rjstruct.c0_rjstruct()
    rj.Rho = 5.0 / 256.0  # the evaluation ROIs carry Poisson(5) emitters
    rj.N_Burnin = rj.N_Trials = jumps
    return rj


def _match_rmse(final_state: np.ndarray, final_n: np.ndarray, n_em: np.ndarray, xyi: np.ndarray, idx) -> tuple:
    from scipy.optimize import linear_sum_assignment
    nmax = (final_state.shape[1] - 4) // 4
    se, cnt = 0.0, 0
    for r in idx:
        k = int(n_em[r])
        if k == 0 or int(final_n[r]) != k:
            continue
        X = final_state[r, 4 + nmax:4 + nmax + k]
        Y = final_state[r, 4 + 2 * nmax:4 + 2 * nmax + k]
        tx, ty = xyi[r, :k, 0], xyi[r, :k, 1]
        d2 = (X[:, None] - tx[None, :]) ** 2 + (Y[:, None] - ty[None, :]) ** 2
        i, j = linear_sum_assignment(d2)
        se += float(d2[i, j].sum())
        cnt += k
    return (float(np.sqrt(se / cnt)) if cnt else float("nan")), cnt


START_COUNTS = (0, 2, 8, 12)   # dispersed start states of the M = 4 chains of a ROI


def dispersed_starts(n: int, seed: int = 11, intensity: float = 1000.0) -> dict:
    """Start states of chain c of ROI r at row c n + r: START_COUNTS[c]
    emitters at uniform positions in the 16x16 ROI, all of `intensity`
    photons (torch CUDA init_n [M n], init_ixy [M n][3][32])."""
    import torch
    M = len(START_COUNTS)
    rng = np.random.default_rng(seed)
    init_n = np.repeat(np.asarray(START_COUNTS, np.int32), n)
    ixy = np.zeros((M * n, 3, 32), np.float32)
    for c, k in enumerate(START_COUNTS):
        if k:
            ixy[c * n:(c + 1) * n, 0, :k] = intensity
            ixy[c * n:(c + 1) * n, 1:, :k] = rng.uniform(0.0, 16.0, size=(n, 2, k))
    return {"init_n": torch.from_numpy(init_n).cuda(), "init_ixy": torch.from_numpy(ixy).cuda()}


def run_arm(s, ev, rj, proposal: str, tables=None, init=None, seed: int = 7, trace: bool = True,
            extra_s: float = 0.0, copies: int = 1):
    """One batched run of `copies` chains per ROI (chain c of ROI r at row
    c n + r, so the chains of one ROI sit in different move-stream groups;
    all rows of a ROI read its pixels and learned tables at offset 256 r);
    init: start states for all rows (or None: empty starts)."""
    import torch
    n0 = int(ev["n_em"].numel())
    n = n0 * copies
    T = rj.N_Burnin + rj.N_Trials
    dev = {"data": ev["data"].reshape(-1),
           "offsets": (torch.arange(n, dtype=torch.int64, device="cuda") % n0) * 256,
           "xsize": torch.full((n,), 16, dtype=torch.int32, device="cuda"),
           "ysize": torch.full((n,), 16, dtype=torch.int32, device="cuda"), "side_max": 16}
    if tables is not None:
        dev["birth_cdf"], dev["birth_sub"] = tables["cdf"], tables["sub"]
    if init is not None:
        dev["init_n"], dev["init_ixy"] = init["init_n"], init["init_ixy"]
    outs = {k: torch.zeros(n, dtype=torch.int32, device="cuda")
            for k in ("map_n", "final_n", "status", "n_entries", "llr_evals")}
    outs["final_state"] = torch.zeros((n, 4 + 4 * 32), dtype=torch.float32, device="cuda")
    if trace:
        outs["n_trace"] = torch.zeros((n, T), dtype=torch.uint8, device="cuda")
        outs["x_trace"] = torch.zeros((n, T), dtype=torch.float32, device="cuda")
    p = rjstruct.mcmc_params(rj)
    bg0 = rjstruct.initial_bg(rj)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=seed, arith="fast", outs=outs,
                 stream=stream.cuda_stream, bg0=bg0, proposal=proposal)
    e1.record(stream)
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3 + extra_s
    assert int((outs["status"] != 0).sum()) == 0
    return outs, secs


def arm_stats(outs, secs, ev_host, subset, copies: int) -> dict:
    """Multi-chain diagnostics over `subset` ROIs (rows c n + r of the
    `copies` chains), accuracy and RMSE from every ROI's first chain."""
    import torch
    n = ev_host["n_em"].shape[0]
    ent = outs["n_entries"].cpu().numpy()
    idx = np.asarray(subset)
    rows = np.concatenate([idx + c * n for c in range(copies)])
    ti = torch.from_numpy(rows).to(outs["n_trace"].device)
    nt = outs["n_trace"].index_select(0, ti).cpu().numpy()
    xt = outs["x_trace"].index_select(0, ti).cpu().numpy()
    k = len(idx)
    groups = np.stack([np.arange(k) + c * k for c in range(copies)], 1)
    mc = ess.multi_chain_ess(nt, xt, ent[rows], groups)
    per_chain_n = np.nan_to_num(mc["ess_n"], nan=0.0) / copies
    per_chain_x = np.nan_to_num(mc["ess_x"], nan=0.0) / copies
    chains_s = n * copies / secs
    map_n = outs["map_n"].cpu().numpy()[:n]
    fs = outs["final_state"].cpu().numpy()[:n]
    fn = outs["final_n"].cpu().numpy()[:n]
    rmse, matched = _match_rmse(fs, fn, ev_host["n_em"], ev_host["xyi"], range(min(n, 10000)))
    rn, rx = mc["rhat_n"], mc["rhat_x"]
    return {"chains_per_s": chains_s, "rois_per_s": n / secs, "seconds": secs, "chains_per_roi": copies,
            "ess_n_per_chain": float(per_chain_n.mean()), "ess_x_per_chain": float(per_chain_x.mean()),
            "ess_n_per_s": float(per_chain_n.mean()) * chains_s, "ess_x_per_s": float(per_chain_x.mean()) * chains_s,
            "rhat_n_median": float(np.nanmedian(rn)) if np.isfinite(rn).any() else float("nan"),
            "rhat_x_median": float(np.nanmedian(rx)) if np.isfinite(rx).any() else float("nan"),
            "rhat_n_above_1_05": float(np.mean(rn[np.isfinite(rn)] > 1.05)) if np.isfinite(rn).any() else 0.0,
            "rhat_x_above_1_05": float(np.mean(rx[np.isfinite(rx)] > 1.05)) if np.isfinite(rx).any() else 0.0,
            "map_count_accuracy": float(np.mean(map_n == np.minimum(ev_host["n_em"], 32))),
            "rmse_px": rmse, "rmse_emitters": matched,
            "ess_subset": int(k), "constant_n_rois": int(np.sum(~np.isfinite(mc["ess_n"])))}


def evaluate(train_rois: int = 2_000_000, batch: int = 1024, n_eval: int = 50_000, jumps: int = 3000,
             ess_subset: int = 2000, net_seed: int = 0, lr: float = 2e-3,
             sweep=(100, 200, 400, 800, 1600)) -> dict:
    """The three arms, M = 4 dispersed chains per ROI each: uniform
    proposals; learned proposals; learned proposals with the first chain
    started from the network's state."""
    import torch
    net = learned.ProposalNet(seed=net_seed)
    steps = max(1, train_rois // batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = net.train(steps, batch=batch, lr=lr, data_seed=1)
    train_s = time.perf_counter() - t0
    ev = learned.generate(n_eval, seed=2024)
    ev_host = {k: v.cpu().numpy() for k, v in ev.items()}
    s = sampler.Sampler()
    # warm-up of the inference path (first launches load the kernels)
    learned.init_states(net.infer(ev["data"][:64]))
    # network inference (and start states) count against the learned arms
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    tables = net.infer(ev["data"])
    e1.record()
    init = learned.init_states(tables)
    e2.record()
    torch.cuda.synchronize()
    infer_s = e0.elapsed_time(e1) / 1e3
    init_s = e1.elapsed_time(e2) / 1e3
    M = len(START_COUNTS)
    starts = dispersed_starts(n_eval)
    net_first = {"init_n": starts["init_n"].clone(), "init_ixy": starts["init_ixy"].clone()}
    net_first["init_n"][:n_eval] = init["init_n"]
    net_first["init_ixy"][:n_eval] = init["init_ixy"]
    rng = np.random.default_rng(0)
    subset = np.sort(rng.choice(n_eval, size=min(ess_subset, n_eval), replace=False))
    arms = {"uniform": dict(proposal="uniform", init=starts),
            "learned": dict(proposal="learned", tables=tables, init=starts, extra_s=infer_s),
            "learned_init": dict(proposal="learned", tables=tables, init=net_first, extra_s=infer_s + init_s)}
    stats = {}
    for name, kw in arms.items():
        out, sec = run_arm(s, ev, _rj(jumps), seed=7, copies=M, **kw)
        stats[name] = arm_stats(out, sec, ev_host, subset, M)
        del out
    # MAP accuracy, RMSE and throughput against chain length (one chain per
    # ROI, the first start state, no traces)
    single = {"uniform": dict(proposal="uniform"),
              "learned": dict(proposal="learned", tables=tables, extra_s=infer_s),
              "learned_init": dict(proposal="learned", tables=tables, init=init, extra_s=infer_s + init_s)}
    curve = {name: [] for name in single}
    for J in tuple(sweep) + (jumps,):
        for name, kw in single.items():
            out, sec = run_arm(s, ev, _rj(J), seed=7, trace=False, **kw)
            acc = float(np.mean(out["map_n"].cpu().numpy() == np.minimum(ev_host["n_em"], 32)))
            rmse, _ = _match_rmse(out["final_state"].cpu().numpy(), out["final_n"].cpu().numpy(), ev_host["n_em"],
                                  ev_host["xyi"], range(min(n_eval, 10000)))
            curve[name].append({"jumps": J, "map_count_accuracy": acc, "rmse_px": rmse, "rois_per_s": n_eval / sec})
    full_u = curve["uniform"][-1]
    target_acc, target_rmse = full_u["map_count_accuracy"], full_u["rmse_px"]
    equal = {}
    for name in ("learned", "learned_init"):
        ok = [c for c in curve[name] if c["map_count_accuracy"] >= target_acc and c["rmse_px"] <= 1.05 * target_rmse]
        if ok:
            best = min(ok, key=lambda c: c["jumps"])
            equal[name] = {**best, "throughput_ratio": best["rois_per_s"] / full_u["rois_per_s"]}
        else:
            equal[name] = None
    u = stats["uniform"]
    return {
        "workload": f"learned vs uniform proposals: {n_eval} fresh 16x16 ROIs, Poisson(5) emitters, "
                    f"{jumps}+{jumps} jumps, {M} dispersed chains per ROI; network trained on {steps * batch} "
                    f"generator ROIs",
        "train_rois": steps * batch, "train_seconds": train_s, "train_rois_per_s": steps * batch / train_s,
        "train_loss_first_last": [float(loss[:50].mean()), float(loss[-50:].mean())],
        "infer_seconds": infer_s, "init_seconds": init_s,
        "arms": stats,
        "ess_n_per_s_ratio": stats["learned"]["ess_n_per_s"] / max(u["ess_n_per_s"], 1e-30),
        "ess_x_per_s_ratio": stats["learned"]["ess_x_per_s"] / max(u["ess_x_per_s"], 1e-30),
        "ess_n_per_s_ratio_init": stats["learned_init"]["ess_n_per_s"] / max(u["ess_n_per_s"], 1e-30),
        "ess_x_per_s_ratio_init": stats["learned_init"]["ess_x_per_s"] / max(u["ess_x_per_s"], 1e-30),
        "accuracy_vs_jumps": curve,
        "equal_accuracy_vs_uniform_at_full_length": {"target_accuracy": target_acc, "target_rmse_px": target_rmse,
                                                     "rmse_tolerance": 0.05, **equal},
    }
