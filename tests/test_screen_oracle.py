"""The pair-screen network's CPU oracle checked on its own (no GPU): its
backward pass against central finite differences of its forward pass, and
its bf16 rounding against hand-worked values."""
import numpy as np

from oracle import screen_mlp as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.3, M.NPARAMS)
    x = rng.normal(0, 1, (64, M.NFEAT))
    y = rng.normal(0, 1, 64)
    _, g, _ = M.forward_backward(w, x, y, round_bf16=False)
    eps = 1e-6
    for q in rng.integers(0, M.NPARAMS, 60):
        wp, wm = w.copy(), w.copy()
        wp[q] += eps
        wm[q] -= eps
        fd = (M.forward_backward(wp, x, y, False)[2] - M.forward_backward(wm, x, y, False)[2]) / (2 * eps)
        assert abs(fd - g[q]) <= 1e-6 * (abs(fd) + 1e-3), q


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -7, -0.0, 65504.0], np.float32)
    assert M.bf16(v).tolist() == [1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, -0.0, 65536.0]
