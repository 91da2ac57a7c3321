"""Birth-proposal tables (host side)."""
import numpy as np
import pytest

from bamf_gb300 import proposal


def test_tables_encode_the_cell_density():
    rng = np.random.default_rng(0)
    X, Y = 5, 3
    cells = rng.gamma(0.5, size=(4 * X, 4 * Y))
    cdf, sub = proposal.tables_from_cells(cells)
    assert cdf.shape == (X * Y,) and sub.shape == (X * Y * 16,)
    assert cdf[-1] == pytest.approx(1.0, abs=1e-6)
    assert np.all(np.diff(cdf) >= 0)
    np.testing.assert_allclose(sub.reshape(-1, 16).sum(1), 1.0, atol=1e-5)
    p = cells / cells.sum()
    for cx, cy in [(0, 0), (3, 11), (19, 5), (7, 2)]:
        x, y = (cx + 0.5) / 4, (cy + 0.5) / 4
        assert proposal.density(cdf, sub, X, Y, x, y) == pytest.approx(p[cx, cy] * 16, rel=1e-4)
    assert proposal.density(cdf, sub, X, Y, -0.1, 1.0) == 0.0
    # integrates to one over the ROI
    xs = (np.arange(4 * X) + 0.5) / 4
    ys = (np.arange(4 * Y) + 0.5) / 4
    tot = sum(proposal.density(cdf, sub, X, Y, x, y) for x in xs for y in ys) / 16
    assert tot == pytest.approx(1.0, rel=1e-4)


def test_batch_tables_checks_shapes():
    with pytest.raises(ValueError):
        proposal.batch_tables([np.ones((8, 8))], [3], [2])
    c, s = proposal.batch_tables([np.ones((8, 8)), np.ones((12, 4))], [2, 3], [2, 1])
    assert c.shape == (4 + 3,) and s.shape == (16 * 7,)
