"""The learned birth proposal on the GPU: synthetic generator, network
forward (birth tables, count logits) and gradients against the torch CPU
oracle (oracle/cnn_torch.py), and training."""
import numpy as np
import pytest

from bamf_gb300 import synth

pytestmark = pytest.mark.gpu


def _host(b):
    return {k: v.cpu().numpy() for k, v in b.items()}


def test_generator_follows_the_forward_model_with_poisson_noise(cuda_lib):
    from bamf_gb300 import learned
    b = _host(learned.generate(3000, seed=7))
    n = b["n_em"]
    assert abs(n.mean() - 5.0) < 0.15 and n.max() <= learned.SYNTH_NMAX
    z = []
    for r in range(3000):
        k = int(n[r])
        X, Y, I = b["xyi"][r, :k, 0], b["xyi"][r, :k, 1], b["xyi"][r, :k, 2]
        assert ((X >= 0) & (X < 16) & (Y >= 0) & (Y < 16)).all()
        lam = synth.model_image(16, 16, X, Y, I, 10.0, 1.3).ravel(order="F")
        z.append((b["data"][r] - lam) / np.sqrt(lam))
        assert (b["xyi"][r, k:] == 0).all()
    z = np.concatenate(z)
    assert abs(z.mean()) < 0.01 and abs(z.var() - 1.0) < 0.02, (z.mean(), z.var())
    allI = np.concatenate([b["xyi"][r, :int(n[r]), 2] for r in range(3000)])
    assert abs(np.median(allI) / 1000.0 - 1) < 0.03
    assert abs(np.log(allI).std() - 0.3) < 0.01
    # the same (seed, index) gives the same ROI
    b2 = _host(learned.generate(10, seed=7, first=5))
    np.testing.assert_array_equal(b2["data"], b["data"][5:15])


def test_forward_matches_the_torch_oracle(cuda_lib):
    import torch

    from bamf_gb300 import learned
    from oracle import cnn_torch
    net = learned.ProposalNet(seed=3)
    b = learned.generate(48, seed=9)
    out = net.infer(b["data"])
    theta = torch.tensor(net.get_params())
    data = b["data"].cpu()
    _, cnt_ref, _ = cnn_torch.forward(theta, data, bf16=True)
    cdf_ref, sub_ref = cnn_torch.birth_tables(theta, data, bf16=True)
    cnt = out["count_logits"].cpu()
    assert torch.allclose(cnt, cnt_ref, rtol=2e-2, atol=2e-2), (cnt - cnt_ref).abs().max()
    cdf = out["cdf"].cpu()
    assert (cdf - cdf_ref).abs().max() < 5e-3
    cdf2 = cdf.reshape(48, 256)
    assert torch.allclose(cdf2[:, -1], torch.ones(48), atol=1e-4)
    assert (cdf2[:, 1:] >= cdf2[:, :-1] - 1e-7).all()
    sub = out["sub"].cpu()
    assert (sub - sub_ref).abs().mean() < 1e-3
    assert torch.allclose(sub.reshape(-1, 16).sum(1), torch.ones(48 * 256), atol=1e-4)


@pytest.mark.parametrize("n", [32, 600])
def test_gradients_match_torch_autograd(cuda_lib, n):
    """n = 600 puts several ROIs on each CTA of the weight-gradient kernel
    (accumulation in TMEM across ROIs, next-ROI prefetch)."""
    import torch

    from bamf_gb300 import learned
    from oracle import cnn_torch
    net = learned.ProposalNet(seed=4)
    b = learned.generate(n, seed=11)
    loss, grad = net.loss_grad(b)
    h = _host(b)
    theta = torch.tensor(net.get_params()).requires_grad_(True)
    L = cnn_torch.loss(theta, torch.tensor(h["data"]), h["n_em"], h["xyi"], bf16=True)
    (g,) = torch.autograd.grad(L, theta)
    assert loss == pytest.approx(L.item(), rel=2e-3)
    g = g.numpy()
    for name, (o, shp) in cnn_torch.OFF.items():
        k = int(np.prod(shp))
        a, r = grad[o:o + k].astype(np.float64), g[o:o + k].astype(np.float64)
        rel = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-12)
        cos = float(a @ r / max(np.linalg.norm(a) * np.linalg.norm(r), 1e-30))
        assert rel < 5e-2 and cos > 0.998, (name, rel, cos)


def test_training_lowers_the_loss_and_finds_the_emitters(cuda_lib):
    from bamf_gb300 import learned, proposal
    net = learned.ProposalNet(seed=5)
    tr = net.train(400, batch=256, lr=2e-3, data_seed=21)
    assert np.isfinite(tr).all()
    assert tr[-20:].mean() < 0.8 * tr[:20].mean(), (tr[:20].mean(), tr[-20:].mean())
    ev = learned.generate(200, seed=99)
    out = net.infer(ev["data"])
    cdf = out["cdf"].cpu().numpy().reshape(200, 256)
    sub = out["sub"].cpu().numpy().reshape(200, 256 * 16)
    h = _host(ev)
    gain = []
    for r in range(200):
        for e in range(int(h["n_em"][r])):
            x, y = h["xyi"][r, e, 0], h["xyi"][r, e, 1]
            gain.append(proposal.density(cdf[r], sub[r], 16, 16, x, y) * 256.0)
    print("mean learned density at the true emitters, relative to uniform:", np.mean(gain))
    assert np.mean(gain) > 5.0


def test_start_states_follow_the_count_logits_and_density(cuda_lib):
    """The network start state: n0 = argmax of the count logits, positions
    at distinct high-density sub-cells; a trained network puts them near the
    true emitters."""
    from bamf_gb300 import learned
    net = learned.ProposalNet(seed=6)
    net.train(300, batch=256, lr=2e-3, data_seed=31)
    ev = learned.generate(300, seed=77)
    tab = net.infer(ev["data"])
    st = learned.init_states(tab, intensity=900.0, max_n=10)
    n0 = st["init_n"].cpu().numpy()
    ixy = st["init_ixy"].cpu().numpy()
    cl = tab["count_logits"].cpu().numpy()
    np.testing.assert_array_equal(n0, np.minimum(cl.argmax(1), 10))
    h = {k: v.cpu().numpy() for k, v in ev.items()}
    near = []
    for r in range(300):
        k = int(n0[r])
        assert (ixy[r, 0, :k] == 900.0).all() and (ixy[r, :, k:] == 0).all()
        X, Y = ixy[r, 1, :k], ixy[r, 2, :k]
        assert ((X > 0) & (X < 16) & (Y > 0) & (Y < 16)).all()
        for a in range(k):
            for b in range(a):
                assert (X[a] - X[b]) ** 2 + (Y[a] - Y[b]) ** 2 >= 1.0 - 1e-5
            m = int(h["n_em"][r])
            if m:
                d = np.min((h["xyi"][r, :m, 0] - X[a]) ** 2 + (h["xyi"][r, :m, 1] - Y[a]) ** 2)
                near.append(d < 0.5 ** 2)
    print("start emitters within 0.5 px of a true one:", np.mean(near))
    assert np.mean(near) > 0.6
    print("count accuracy of the start state:", np.mean(n0 == np.minimum(h["n_em"], 10)))


def test_training_on_accepted_states_adapts_to_data_the_generator_misdescribes(cuda_lib):
    """The network learns from states the sampler accepted.  Trained on
    generator ROIs of PSF sigma 1.3 and median intensity 1000, it meets ROIs
    of sigma 1.7 and median 600.  The uniform-birth sampler (given the true
    PSF) runs on 16k of those ROIs; one accepted state per ROI from the
    trial phase becomes a training example (no ground truth is used) and the
    network is fine-tuned on them (bamf_cnn_train_examples).  On fresh
    shifted ROIs the fine-tuned network's loss on the true emitters falls
    and its count head is right more often."""
    import torch
    from bamf_gb300 import learned, mapfit, rjstruct, sampler
    net = learned.ProposalNet(seed=3)
    net.train(300, batch=512, lr=2e-3, data_seed=5, mean_n=5.0, sigma=1.3, i_median=1000.0, i_logsd=0.3,
              bg=10.0)
    shift = dict(mean_n=5.0, sigma=1.7, i_median=600.0, i_logsd=0.3, bg=10.0)
    n = 16384
    tr = learned.generate(n, seed=77, **shift)
    rj = rjstruct.c0_rjstruct()
    rj.Rho = 5.0 / 256.0
    rj.PSF_Sigma = 1.7
    rj.N_Burnin = rj.N_Trials = 1000
    p = rjstruct.mcmc_params(rj)
    pos_len = 64
    thin = mapfit.thinning(2000, pos_len)
    dev = {"data": tr["data"].reshape(-1), "offsets": torch.arange(n, dtype=torch.int64, device="cuda") * 256,
           "xsize": torch.full((n,), 16, dtype=torch.int32, device="cuda"),
           "ysize": torch.full((n,), 16, dtype=torch.int32, device="cuda"), "side_max": 16}
    outs = {k: torch.zeros(n, dtype=torch.int32, device="cuda") for k in ("status", "n_entries")}
    outs["pos_trace"] = torch.zeros((n, pos_len, mapfit.POS_RECORD), dtype=torch.float32, device="cuda")
    outs["pos_thin"] = thin
    sampler.Sampler().run_device(dev, p, rj.P_Offset, rj.P_EmPhotons, rj.P_BgEmPhotons, seed=11, arith="fast",
                                 outs=outs, bg0=rjstruct.initial_bg(rj), proposal="uniform")
    torch.cuda.synchronize()
    assert int((outs["status"] != 0).sum()) == 0
    ex = learned.examples_from_states(tr["data"], outs["pos_trace"], outs["n_entries"], thin, seed=1)
    agree = float((ex["n_em"] == tr["n_em"].clamp(max=16)).float().mean())
    ev = learned.generate(4096, seed=99, **shift)

    def score():
        loss, _ = net.loss_grad(ev)
        cnt = net.infer(ev["data"])["count_logits"].argmax(dim=1)
        acc = float((cnt == ev["n_em"].clamp(max=10).to(cnt.dtype)).float().mean())
        return loss, acc

    loss_a, acc_a = score()
    trace = net.train_examples(ex, steps=300, batch=512, lr=1e-3)
    loss_b, acc_b = score()
    print(f"sampler states match the true count on {agree:.3f} of ROIs; loss {loss_a:.3f} -> {loss_b:.3f}, "
          f"count accuracy {acc_a:.3f} -> {acc_b:.3f}; example loss {trace[0]:.3f} -> {trace[-1]:.3f}")
    assert np.isfinite(trace).all()
    assert loss_b < loss_a - 0.05
    assert acc_b > acc_a
