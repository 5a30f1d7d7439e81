"""The FP64 MLP oracle against central finite differences (CPU only)."""
import numpy as np

from oracle import mlp as omlp


def test_oracle_mlp_gradient_finite_differences():
    d0, h = 7, 9
    rng = np.random.default_rng(0)
    p = rng.standard_normal(h * d0 + h + h * h + h + h + 1) * 0.5
    x = rng.standard_normal((13, d0))
    y = rng.standard_normal(13)
    _, g = omlp.loss_grad(p, x, y, d0, h)
    fd = np.empty_like(p)
    for i in range(p.size):
        e = np.zeros_like(p); e[i] = 1e-6
        fd[i] = (omlp.loss_grad(p + e, x, y, d0, h)[0] - omlp.loss_grad(p - e, x, y, d0, h)[0]) / 2e-6
    assert np.abs(g - fd).max() <= 1e-6 * max(1.0, np.abs(g).max())


def test_oracle_adam_reduces_loss():
    d0, h = 5, 8
    rng = np.random.default_rng(1)
    p = rng.standard_normal(h * d0 + h + h * h + h + h + 1) * 0.3
    x = rng.standard_normal((40, d0))
    y = np.sin(x[:, 0]) + x[:, 1] ** 2
    l0 = omlp.loss_grad(p, x, y, d0, h)[0]
    _, l1 = omlp.adam_train(p, x, y, d0, h, epochs=200, lr=1e-2)
    assert l1 < 0.3 * l0
