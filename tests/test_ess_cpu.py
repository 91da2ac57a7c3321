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
