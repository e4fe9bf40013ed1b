"""The FP64 network oracle (oracle/mlp.py) against finite differences, with its
FP16 roundings switched off: its analytic gradients are right."""
import numpy as np

from oracle import mlp


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(0)
    params = rng.uniform(-0.2, 0.2, mlp.N_PARAMS)
    x = rng.random((64, 7))
    t = rng.random((64, 3))
    mlp.ROUND_FP16 = False
    try:
        _, g = mlp.loss_and_grads(params, x, t)
        # the loss treats y^2 + 0.01 as a constant (stop-gradient): difference that form
        def loss_sg(p, y0):
            y, _ = mlp.forward(p, x)
            return np.mean((y - t) ** 2 / (y0 * y0 + 0.01))
        y0, _ = mlp.forward(params, x)
        idx = rng.choice(mlp.N_PARAMS, 60, replace=False)
        for i in idx:
            e = np.zeros_like(params)
            e[i] = 1e-6
            fd = (loss_sg(params + e, y0) - loss_sg(params - e, y0)) / 2e-6
            assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
    finally:
        mlp.ROUND_FP16 = True
