"""The CPU oracle of the surrogate network: its analytic FP64 backward
agrees with central finite differences."""
import numpy as np

from oracle import mlp_oracle as M


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.1, M.NPARAMS)
    X = rng.normal(size=(16, M.IN))
    T = rng.normal(size=(16, M.OUT))
    _, g = M.loss_grad(p, X, T)
    for i in rng.choice(M.NPARAMS, 60, replace=False).tolist() + [M.OFF_B, M.NPARAMS - 1, M.OFF_W4]:
        h = 1e-6
        q = p.copy()
        q[i] += h
        lp, _ = M.loss_grad(q, X, T)
        q[i] -= 2 * h
        lm, _ = M.loss_grad(q, X, T)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-5, 65504.0], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.0e-5) / 3.0e-5 < 4e-3
