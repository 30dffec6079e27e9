"""The CPU model of the proposer network (oracle/mlp_ref.py) against finite
differences of its own loss (no GPU)."""
import numpy as np

import mlp_ref


def test_cpu_model_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    sizes = [int(np.prod(s)) for s in mlp_ref.SHAPES]
    w = np.concatenate([rng.normal(0, 0.05, n) for n in sizes])
    xa = (rng.random((6, 512)) < 0.3).astype(np.float64)
    xb = (rng.random((6, 512)) < 0.3).astype(np.float64)
    t = rng.random(6)
    loss, g = mlp_ref.loss_grad(w, xa, xb, t)
    idx = np.concatenate([rng.choice(np.arange(o, o + n), 8, replace=False)
                          for o, n in zip(np.cumsum([0] + sizes[:-1]), sizes)])
    eps = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        num = (mlp_ref.loss_grad(wp, xa, xb, t)[0] - mlp_ref.loss_grad(wm, xa, xb, t)[0]) / (2 * eps)
        assert abs(num - g[i]) <= 1e-5 * max(1.0, abs(num)), (i, num, g[i])
