"""Pin the CNN oracle: its autograd gradient against central finite
differences in float64 (CPU only)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import cnn as N


def _params(rng):
    n = sum(27 * a * b + b for a, b in N.SPEC)
    return rng.standard_normal(n) * 0.1


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    grid = (5, 3, 3)                       # (nx, ny, nz) of the level-1 node grid
    nn = 5 * 3 * 3
    p = _params(rng)
    x0 = rng.standard_normal((nn, 7))
    t = rng.standard_normal((nn, 3))
    loss, g, _ = N.loss_and_grad(p, x0, t, grid)
    for i in rng.choice(p.size, 25, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _, _ = N.loss_and_grad(pp, x0, t, grid)
        lm, _, _ = N.loss_and_grad(pm, x0, t, grid)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_oracle_pool_and_upsample_shapes():
    x = torch.ones((1, 2, 5, 9, 5), dtype=torch.float64)
    p = N._pool(x)
    assert tuple(p.shape[2:]) == (3, 5, 3)
    assert torch.allclose(p, torch.ones_like(p))      # average of present children
    u = N._up(p, (5, 9, 5))
    assert tuple(u.shape[2:]) == (5, 9, 5)
