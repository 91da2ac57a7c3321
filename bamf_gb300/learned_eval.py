"""Learned vs uniform birth proposal on 16x16 ROIs: throughput, effective
samples per second, MAP emitter-count accuracy and localisation error.

Protocol (all on one GPU):
  1. train the proposal network on `train_rois` generator ROIs (Poisson(5)
     emitters, the plain-RJMCMC generator otherwise);
  2. draw `n_eval` fresh ROIs from the same generator (another seed);
  3. run the batched fast sampler with UNIFORM and with LEARNED births
     (birth tables from the network; its inference time counts against the
     learned arm), each recording the per-entry emitter-count and mean-X
     traces;
  4. ESS (Geyer initial monotone sequence, bamf_gb300.ess) of both traces
     over the second half of every chain's entries (the trial phase: burn-in
     and trials have the same number of jumps) on a subset of ROIs, scaled
     to ESS/s with the arm's ROIs/s;
  5. MAP emitter-count accuracy over all ROIs, and the localisation RMSE of
     the final state's emitters matched to the truth (Hungarian matching on
     ROIs whose final count equals the true count).
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


def run_arm(s, ev, rj, proposal: str, tables=None, init=None, seed: int = 7, trace: bool = True,
            extra_s: float = 0.0):
    import torch
    n = int(ev["n_em"].numel())
    T = rj.N_Burnin + rj.N_Trials
    dev = {"data": ev["data"].reshape(-1), "offsets": torch.arange(n, dtype=torch.int64, device="cuda") * 256,
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


def arm_stats(outs, secs, ev_host, subset) -> dict:
    n = ev_host["n_em"].shape[0]
    ent = outs["n_entries"].cpu().numpy()
    import torch
    idx = np.asarray(subset)
    ti = torch.from_numpy(idx).to(outs["n_trace"].device)
    nt = outs["n_trace"].index_select(0, ti).cpu().numpy()
    xt = outs["x_trace"].index_select(0, ti).cpu().numpy()
    e = ess.batch_ess(nt, xt, ent[idx], ent[idx] // 2)
    mean_n = float(np.nanmean(np.nan_to_num(e["ess_n"], nan=0.0)))
    mean_x = float(np.nanmean(np.nan_to_num(e["ess_x"], nan=0.0)))
    rois_s = n / secs
    map_n = outs["map_n"].cpu().numpy()
    fs = outs["final_state"].cpu().numpy()
    fn = outs["final_n"].cpu().numpy()
    rmse, matched = _match_rmse(fs, fn, ev_host["n_em"], ev_host["xyi"], range(min(n, 10000)))
    return {"rois_per_s": rois_s, "seconds": secs, "ess_n_per_roi": mean_n, "ess_x_per_roi": mean_x,
            "ess_n_per_s": mean_n * rois_s, "ess_x_per_s": mean_x * rois_s,
            "map_count_accuracy": float(np.mean(map_n == np.minimum(ev_host["n_em"], 32))),
            "rmse_px": rmse, "rmse_emitters": matched,
            "ess_subset": int(len(idx)), "constant_n_chains": int(np.sum(~np.isfinite(e["ess_n"])))}


def evaluate(train_rois: int = 2_000_000, batch: int = 1024, n_eval: int = 50_000, jumps: int = 3000,
             ess_subset: int = 4000, net_seed: int = 0, lr: float = 2e-3,
             sweep=(100, 200, 400, 800, 1600)) -> dict:
    """The three arms: uniform births from an empty start; learned births
    from an empty start; learned births from the network's start state."""
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
    rng = np.random.default_rng(0)
    subset = np.sort(rng.choice(n_eval, size=min(ess_subset, n_eval), replace=False))
    arms = {"uniform": dict(proposal="uniform"),
            "learned": dict(proposal="learned", tables=tables, extra_s=infer_s),
            "learned_init": dict(proposal="learned", tables=tables, init=init, extra_s=infer_s + init_s)}
    stats = {}
    for name, kw in arms.items():
        out, sec = run_arm(s, ev, _rj(jumps), seed=7, **kw)
        stats[name] = arm_stats(out, sec, ev_host, subset)
        del out
    # MAP accuracy and throughput against chain length (no traces)
    curve = {name: [] for name in arms}
    for J in sweep:
        for name, kw in arms.items():
            out, sec = run_arm(s, ev, _rj(J), seed=7, trace=False, **kw)
            acc = float(np.mean(out["map_n"].cpu().numpy() == np.minimum(ev_host["n_em"], 32)))
            curve[name].append({"jumps": J, "map_count_accuracy": acc, "rois_per_s": n_eval / sec})
    for name in arms:
        curve[name].append({"jumps": jumps, "map_count_accuracy": stats[name]["map_count_accuracy"],
                            "rois_per_s": stats[name]["rois_per_s"]})
    target = stats["uniform"]["map_count_accuracy"]
    equal = {}
    for name in ("learned", "learned_init"):
        ok = [c for c in curve[name] if c["map_count_accuracy"] >= target]
        if ok:
            best = min(ok, key=lambda c: c["jumps"])
            equal[name] = {"jumps": best["jumps"], "rois_per_s": best["rois_per_s"],
                           "throughput_ratio": best["rois_per_s"] / stats["uniform"]["rois_per_s"]}
        else:
            equal[name] = None
    return {
        "workload": f"learned vs uniform birth proposal: {n_eval} fresh 16x16 ROIs, Poisson(5) emitters, "
                    f"{jumps}+{jumps} jumps; network trained on {steps * batch} generator ROIs",
        "train_rois": steps * batch, "train_seconds": train_s, "train_rois_per_s": steps * batch / train_s,
        "train_loss_first_last": [float(loss[:50].mean()), float(loss[-50:].mean())],
        "infer_seconds": infer_s, "init_seconds": init_s,
        "arms": stats,
        "ess_n_per_s_ratio": stats["learned"]["ess_n_per_s"] / max(stats["uniform"]["ess_n_per_s"], 1e-30),
        "ess_x_per_s_ratio": stats["learned"]["ess_x_per_s"] / max(stats["uniform"]["ess_x_per_s"], 1e-30),
        "accuracy_vs_jumps": curve,
        "equal_accuracy_vs_uniform_at_full_length": {"target_accuracy": target, **equal},
    }
