"""The NumPy reference of the radiance-cache MLP is itself checked: its
analytic gradient against central finite differences in float64 (CPU)."""
import numpy as np

import nrc_reference as ref


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n = 24
    q = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3)),
                        rng.uniform(0.1, 0.9, (n, 3))], 1)
    q[:, 3:6] /= np.linalg.norm(q[:, 3:6], axis=1, keepdims=True)
    x0 = ref.encode(q, np.zeros(3), np.ones(3)).astype(np.float64)
    w = rng.uniform(-0.3, 0.3, 17408)
    target = rng.uniform(0, 2, (n, 3))
    loss, _, g = ref.loss_and_grad(x0, w, target, fp16=False)
    idx = np.concatenate([rng.integers(0, 4096, 6), 4096 * 2 + rng.integers(0, 4096, 6),
                          4 * 4096 + rng.integers(0, 64, 6) * 16 + rng.integers(0, 3, 6)])
    for i in idx:
        e = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += e
        wm[i] -= e
        # the relative loss treats the denominator as a constant: freeze it
        fd = (_loss_frozen(x0, wp, target, w) - _loss_frozen(x0, wm, target, w)) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])
    assert loss > 0


def _loss_frozen(x0, w, target, w_den):
    _, out = ref.forward(x0, w, fp16=False)
    _, out_d = ref.forward(x0, w_den, fp16=False)
    p, pd = out[:, :3], out_d[:, :3]
    return float(((p - target) ** 2 / (pd * pd + 0.01)).mean())
