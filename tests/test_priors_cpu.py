"""Prior construction statistics (bamf_gb300.priors) against scipy's
implementations of the same definitions (MATLAB's fitdist / gamfit / gammainc
are not available here: parity with them is unpinned)."""
import numpy as np
import pytest

scipy = pytest.importorskip("scipy")

from bamf_gb300 import priors  # noqa: E402


def test_kernel_pdf_matches_scipy_gaussian_kde_with_fixed_bandwidth():
    from scipy.stats import gaussian_kde
    x = np.random.default_rng(0).lognormal(np.log(1500), 0.3, 3000)
    grid = np.arange(0, 5000, 10.0)
    k = gaussian_kde(x, bw_method=75.0 / x.std(ddof=1))
    np.testing.assert_allclose(priors.kernel_pdf(x, 75.0, grid), k(grid), rtol=1e-9, atol=1e-15)


def test_gamma_fit_matches_scipy_mle():
    from scipy.stats import gamma
    x = np.random.default_rng(1).gamma(4.5, 6.0, 5000)
    a, b = priors.gamma_fit(x)
    a0, _, b0 = gamma.fit(x, floc=0)
    assert a == pytest.approx(a0, rel=1e-5) and b == pytest.approx(b0, rel=1e-5)
    g = np.arange(0, 100, 0.5)
    np.testing.assert_allclose(priors.gamma_pdf(g, a, b), gamma.pdf(g, a, scale=b), rtol=1e-10, atol=1e-300)


def test_p_value_is_the_chi_square_tail():
    from scipy.stats import chi2
    LL = -np.array([10.0, 30.0, 60.0, 100.0])
    # the reference forms 1 - gammainc(...): same cancellation in the far tail
    np.testing.assert_allclose(priors.p_value("Basic", 8, LL), chi2.sf(-2 * LL, 60), rtol=1e-10, atol=1e-15)


def test_threhs_sma_applies_every_cut():
    SMD = {"X": np.array([1.0, 4.0, 9.0, 3.0, 3.0, 3.0]), "Y": np.array([1.0, 4.0, 3.0, 3.0, 3.0, 3.0]),
           "X_SE": np.array([0.1, 0.1, 0.1, 0.3, 0.1, 0.1]), "Y_SE": np.full(6, 0.1),
           "Photons": np.array([500.0, 800.0, 900.0, 900.0, 50.0, 900.0]),
           "BG": np.array([10.0, 10.0, 10.0, 10.0, 10.0, -1.0]), "LogLikelihood": np.full(6, -30.0)}
    r = priors.threhsSMA(SMD, {"MinPValue": 0.01, "MinPhotons": 100}, 8)
    np.testing.assert_array_equal(r["Photons"], [500.0, 800.0])


def test_signal_prior_trims_a_second_mode():
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.normal(1500, 150, 4000), rng.normal(4000, 150, 400)])
    pdf, grid, kept = priors.signal_prior(x, 10.0)
    assert kept.max() < 3500 and len(kept) < len(x)
    assert abs(pdf.sum() * 10.0 - 1.0) < 1e-3
    assert grid[0] == 0 and grid[1] == 10.0
