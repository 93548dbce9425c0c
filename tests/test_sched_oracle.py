"""The scheduler MLP's CPU oracle is pinned by finite differences (no GPU)."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(size=mlp.N_PARAMS) * 0.2
    X = rng.normal(size=(9, mlp.IN))
    T = rng.normal(size=9)
    loss, g = mlp.loss_grad(p, X, T)
    assert g.shape == (mlp.N_PARAMS,)
    eps = 1e-6
    for i in rng.integers(0, mlp.N_PARAMS, 64):
        q = p.copy()
        q[i] += eps
        lp, _ = mlp.loss_grad(q, X, T)
        q[i] -= 2 * eps
        lm, _ = mlp.loss_grad(q, X, T)
        assert abs((lp - lm) / (2 * eps) - g[i]) < 1e-7 * max(1.0, abs(g[i]))
    y, _ = mlp.forward(p, X)
    assert np.isclose(loss, np.mean((y - T) ** 2))


def test_parameter_count_matches_the_abi_header():
    import re
    import os
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "bsgpu.h")).read()
    assert int(re.search(r"#define BSG_SCHED_FEATURES (\d+)", hdr).group(1)) == mlp.IN
