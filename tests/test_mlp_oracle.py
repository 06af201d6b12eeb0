"""The numpy MLP oracle itself: finite differences agree with its gradients
(float64, no rounding), and its bf16 rounding matches torch's."""
import numpy as np


def test_oracle_gradients_finite_differences():
    from oracle import mlp_oracle as M
    rng = np.random.default_rng(0)
    D, O, P, B = 32, 16, 15, 7
    npar = D * M.H + M.H + M.H * M.H + M.H + M.H * O + O
    w = rng.normal(0, 0.1, npar)
    X = rng.normal(0, 1, (B, D))
    y = rng.integers(0, P, B)
    y[2] = -1
    loss, g = M.loss_and_grads(w, D, O, P, X, y, rounding=False)
    for idx in rng.choice(npar, 40, replace=False):
        e = np.zeros(npar)
        e[idx] = 1e-6
        lp, _ = M.loss_and_grads(w + e, D, O, P, X, y, rounding=False)
        lm, _ = M.loss_and_grads(w - e, D, O, P, X, y, rounding=False)
        fd = (lp - lm) / 2e-6 / B
        assert abs(fd - g[idx]) < 1e-6 + 1e-4 * abs(fd), (idx, fd, g[idx])


def test_bf16_rounding_matches_torch():
    import torch
    from oracle import mlp_oracle as M
    x = np.random.default_rng(1).normal(0, 3, 10000).astype(np.float32)
    x[:4] = [1.00390625, 1.01171875, -2.5, 0.0]  # ties
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(M.bf16(x).astype(np.float32), want)
