"""The MLP oracle's analytic gradient against central finite differences
(in float64 with the BF16 roundings switched off, so the loss is smooth)."""
from __future__ import annotations

import numpy as np

from conftest import ROOT  # noqa: F401  (puts oracle/ on the path)
import mlp_oracle as M  # noqa: E402


def test_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(M, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.default_rng(0)
    theta = M.init(1).astype(np.float64) + 0.05 * rng.standard_normal(M.N_PARAMS)
    x = rng.standard_normal((7, 16))
    y = rng.integers(0, M.N_CLASSES, 7)
    _, g = M.loss_and_grad(theta, x, y)
    for i in rng.choice(M.N_PARAMS, 60, replace=False):
        e = np.zeros(M.N_PARAMS)
        e[i] = 1e-6
        lp, _ = M.loss_and_grad(theta + e, x, y)
        lm, _ = M.loss_and_grad(theta - e, x, y)
        assert abs((lp - lm) / 2e-6 - g[i]) <= 1e-6 + 1e-5 * abs(g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0], np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5 and r[4] == 0.0
