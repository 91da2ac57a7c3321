"""The learned proposal's gradient oracle (CPU): the torch statement of the
network and loss against FP64 central finite differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import cnn_torch  # noqa: E402


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    data = rng.poisson(10 + 200 * rng.random((n, 256))).astype(np.float64)
    n_em = rng.integers(0, 6, size=n).astype(np.int32)
    xyi = np.zeros((n, 16, 3))
    xyi[:, :, :2] = rng.uniform(0, 16, size=(n, 16, 2))
    return torch.tensor(data), n_em, xyi


def test_parameter_layout_covers_the_vector():
    ends = sorted((o, o + int(np.prod(s))) for o, s in cnn_torch.OFF.values())
    assert ends[0][0] == 0 and ends[-1][1] == cnn_torch.NPARAM
    assert all(a[1] == b[0] for a, b in zip(ends, ends[1:]))


def test_autograd_matches_fp64_finite_differences():
    torch.manual_seed(0)
    theta = (0.1 * torch.randn(cnn_torch.NPARAM, dtype=torch.float64)).requires_grad_(True)
    data, n_em, xyi = _batch(3, 1)
    L = cnn_torch.loss(theta, data, n_em, xyi, bf16=False)
    (g,) = torch.autograd.grad(L, theta)
    rng = np.random.default_rng(2)
    eps = 1e-6
    for k in range(4):
        v = torch.tensor(rng.standard_normal(cnn_torch.NPARAM))
        v = v / v.norm()
        with torch.no_grad():
            lp = cnn_torch.loss(theta + eps * v, data, n_em, xyi, bf16=False)
            lm = cnn_torch.loss(theta - eps * v, data, n_em, xyi, bf16=False)
        fd = (lp - lm).item() / (2 * eps)
        an = float(g @ v)
        assert fd == pytest.approx(an, rel=1e-5, abs=1e-9), (k, fd, an)


def test_birth_tables_are_normalised():
    theta = 0.1 * torch.randn(cnn_torch.NPARAM, dtype=torch.float64)
    data, _, _ = _batch(2, 3)
    cdf, sub = cnn_torch.birth_tables(theta, data, bf16=False)
    cdf = cdf.reshape(2, 256)
    assert torch.allclose(cdf[:, -1], torch.ones(2, dtype=torch.float64))
    assert torch.allclose(sub.reshape(-1, 16).sum(1), torch.ones(512, dtype=torch.float64))
