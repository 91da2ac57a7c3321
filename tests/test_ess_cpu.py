"""ESS estimator (Geyer initial monotone sequence) on chains of known ESS."""
import numpy as np
import pytest

from bamf_gb300 import ess


def _ar1(n, rho, seed):
    rng = np.random.default_rng(seed)
    e = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = e[0] / np.sqrt(1 - rho * rho)
    for i in range(1, n):
        x[i] = rho * x[i - 1] + e[i]
    return x


@pytest.mark.parametrize("rho", [0.0, 0.5, 0.9, 0.99])
def test_ar1_ess_matches_theory(rho):
    n = 200_000
    x = _ar1(n, rho, 1)
    want = n * (1 - rho) / (1 + rho)
    got = ess.ess_geyer(x)
    assert abs(got / want - 1) < 0.15, (got, want)


def test_autocov_matches_direct_sum():
    x = np.random.default_rng(2).standard_normal(500)
    g = ess.autocov(x)
    d = x - x.mean()
    for k in (0, 1, 7, 100):
        assert g[k] == pytest.approx(np.dot(d[:500 - k], d[k:]) / 500, rel=1e-9, abs=1e-12)


def test_constant_and_short_chains_are_nan():
    assert np.isnan(ess.ess_geyer(np.ones(100)))
    assert np.isnan(ess.ess_geyer(np.arange(3.0)))


def test_batch_ess_uses_entries_after_burnin_and_fills_nan():
    rng = np.random.default_rng(3)
    k, T = 3, 4000
    n_trace = rng.integers(0, 4, size=(k, T)).astype(np.uint8)
    x_trace = rng.uniform(0, 16, size=(k, T)).astype(np.float32)
    x_trace[:, ::7] = np.nan
    n_entries = np.array([4000, 3000, 10])
    r = ess.batch_ess(n_trace, x_trace, n_entries, 1000)
    assert list(r["length"]) == [3000, 2000, 0]
    assert np.isnan(r["ess_n"][2])
    # i.i.d. traces: ESS close to the chain length
    assert abs(r["ess_n"][0] / 3000 - 1) < 0.2
    assert abs(r["ess_x"][1] / 2000 - 1) < 0.25
    s = ess.summarize(r, 2.0)
    assert s["ess_n_per_s"] == pytest.approx(np.nansum(r["ess_n"]) / 2.0)


def _ar1_chains(phi, n, m, rng, shift=None):
    x = np.zeros((m, n))
    e = rng.normal(size=(m, n))
    for t in range(1, n):
        x[:, t] = phi * x[:, t - 1] + e[:, t]
    return x if shift is None else x + np.asarray(shift, float)[:, None]


def test_multi_chain_bulk_ess_matches_ar1_theory():
    """Four AR(1) chains: the bulk ESS (split, rank-normalised, multi-chain
    Geyer) averages to M N (1 - phi) / (1 + phi) within 10%, and R-hat is
    within 1.01 of 1."""
    rng = np.random.default_rng(3)
    phi, n, m = 0.8, 3000, 4
    vals, rh = [], []
    for _ in range(20):
        c = _ar1_chains(phi, n, m, rng)
        vals.append(ess.ess_bulk(c))
        rh.append(ess.rhat(c))
    want = m * n * (1 - phi) / (1 + phi)
    assert abs(np.mean(vals) / want - 1) < 0.1, (np.mean(vals), want)
    assert max(rh) < 1.01


def test_unmixed_chains_get_high_rhat_and_small_ess():
    """Chains stuck in different modes: R-hat far above 1, ESS of the order
    of the number of chains - what one chain's own ESS cannot show."""
    rng = np.random.default_rng(4)
    c = _ar1_chains(0.5, 2000, 4, rng, shift=[0, 0, 6, 6])
    assert ess.rhat(c) > 1.3
    assert ess.ess_bulk(c) < 50
    assert min(ess.ess_geyer(x) for x in c) > 500


def test_multi_chain_ess_groups_rows_and_handles_missing_positions():
    rng = np.random.default_rng(5)
    T = 400
    n_trace = rng.integers(2, 5, size=(8, T)).astype(np.uint8)
    x_trace = rng.normal(8.0, 0.1, size=(8, T)).astype(np.float32)
    x_trace[0, 300:310] = np.nan
    out = ess.multi_chain_ess(n_trace, x_trace, np.full(8, T), np.array([[0, 2, 4, 6], [1, 3, 5, 7]]))
    assert np.all(np.isfinite(out["ess_n"])) and np.all(np.isfinite(out["ess_x"]))
    assert np.all(out["rhat_n"] < 1.05) and np.all(out["ess_x"] > 100)
