"""CPU checks of the numpy MLP reference (test infrastructure): its analytic gradient matches
central finite differences, and BF16 rounding is round-to-nearest-even."""
import numpy as np

import mlp_ref


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159265], np.float32)
    r = mlp_ref.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5 and abs(r[4] - 3.140625) < 1e-12


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    din, h, dout, B = 7, 6, 5, 9
    n = h * din + h + h * h + h + dout * h + dout
    # weights already on the BF16 grid so the straight-through gradient is the true gradient
    w = mlp_ref.bf16_round(rng.standard_normal(n).astype(np.float32) * 0.5)
    X = rng.standard_normal((B, din))
    T = rng.standard_normal((B, dout))
    loss, g, _ = mlp_ref.loss_grad(w, X, T, din, h, dout)
    # finite differences on the biases (not rounded) and on the activations path
    offs = [h * din, h * din + h + h * h, h * din + h + h * h + h + dout * h]
    for o in offs:
        for j in range(3):
            e = np.zeros(n)
            e[o + j] = 1e-6
            lp, _, _ = mlp_ref.loss_grad(w + e, X, T, din, h, dout)
            lm, _, _ = mlp_ref.loss_grad(w - e, X, T, din, h, dout)
            fd = (lp - lm) / 2e-6
            assert abs(fd - g[o + j]) <= 1e-6 * max(1.0, abs(fd))
