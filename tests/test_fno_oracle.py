"""The FP64 FNO oracle: its hand-written backward pass against central finite differences
(CPU).  The GPU forward/backward kernels are checked against this oracle in the GPU tests."""
from __future__ import annotations

import numpy as np

from oracle import fno


def test_fno_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    modes, layers = 2, 2
    p = fno.init_params(3, 3, width=4, modes=modes, layers=layers, hidden=6, seed=1)
    for k in p:
        if k.endswith("_b") or k.startswith("b"):
            p[k] = 0.1 * rng.standard_normal(p[k].shape)
    a = rng.standard_normal((2, 3, 8, 12))
    target = rng.standard_normal((2, 3, 8, 12))

    def loss(params):
        out, _ = fno.forward(params, a, modes, layers)
        return fno.mse(out, target)[0]

    out, cache = fno.forward(p, a, modes, layers)
    _, dout = fno.mse(out, target)
    grads = fno.backward(p, cache, dout, modes, layers)
    eps = 1e-6
    for name, value in p.items():
        flat = value.reshape(-1)
        for idx in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + eps
            up = loss(p)
            flat[idx] = old - eps
            down = loss(p)
            flat[idx] = old
            fd = (up - down) / (2 * eps)
            an = grads[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (name, idx, fd, an)
