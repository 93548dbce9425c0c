"""Learned Strassen scheduler: the device forward / backward kernels against
the CPU oracle, training, node features, the per-node options (Strassen
depth 1-3, dense tile) reaching the recursion, and a network trained on
nodes of every level evaluated against every fixed policy."""
import numpy as np
import pytest

from oracle import mlp
from strassen_gb300 import sched as SC

pytestmark = pytest.mark.gpu


def test_gradients_match_oracle(api, ctx):
    net = api.StrassenScheduler(ctx, seed=3)
    rng = np.random.default_rng(1)
    p = (rng.normal(size=net.n_params) * 0.15).astype(np.float32)
    net.params = p
    X = rng.normal(size=(37, api.SCHED_FEATURES)).astype(np.float32)
    T = rng.normal(size=37).astype(np.float32)
    loss, g = net.loss_grad(X, T)
    lo, go = mlp.loss_grad(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - lo) <= 1e-5 * max(1.0, lo)
    assert np.linalg.norm(g - go) <= 1e-5 * np.linalg.norm(go)
    y = net.predict(X)
    yo, _ = mlp.forward(p.astype(np.float64), X.astype(np.float64))
    assert np.max(np.abs(y - yo)) <= 1e-5 * max(1.0, np.max(np.abs(yo)))


def test_training_fits_a_known_function(api, ctx):
    net = api.StrassenScheduler(ctx, seed=5)
    rng = np.random.default_rng(2)
    X = rng.uniform(-1, 1, size=(512, api.SCHED_FEATURES)).astype(np.float32)
    T = (np.tanh(2 * X[:, 4]) - 0.5 * X[:, 6] + 0.3 * X[:, 9] * X[:, 17]).astype(np.float32)
    l0, _ = net.loss_grad(X, T)
    lf = net.train(X, T, epochs=150, batch=64, lr=3e-3, seed=1)
    l1, _ = net.loss_grad(X, T)
    assert l1 < 0.05 * l0, (l0, lf, l1)
    # deterministic: the same seed and data give the same parameters
    net2 = api.StrassenScheduler(ctx, seed=5)
    net2.train(X, T, epochs=150, batch=64, lr=3e-3, seed=1)
    assert np.array_equal(net.params, net2.params)


def test_root_features(api, ctx):
    spec = (16, 64, 1.0, 3.0, 1e-10, 11)  # fully dense core
    _, _, gA, gB, gC = SC.build(spec, ctx)
    gC.fill_with_values(0.0)
    f, ok = api.strassen_root_features(gC, gA, gB, spec[4])
    assert ok
    assert f[6] == 1.0 and f[7] == 1.0 and f[8] == 1.0  # densities
    assert abs(f[9:17].sum() - 1.0) < 1e-6 and abs(f[17:25].sum() - 1.0) < 1e-6  # histograms
    assert abs(f[1] - np.log2(16) / 8) < 1e-6
    gC2 = api.BlockSparseMatrix(1024, 1024, 64, 64, 0.0, ctx=ctx)  # C not allocated: not eligible
    f2, ok2 = api.strassen_root_features(gC2, gA, gB, spec[4])
    assert not ok2


@pytest.mark.parametrize("policy", ["none", "root", "cost", "dense"])
def test_policies_give_the_product(api, ctx, policy):
    spec = (16, 64, 0.5, 2.0, 1e-9, 21)
    A, B, gA, gB, gC = SC.build(spec, ctx)
    pol = {"none": api.SCHED_NONE, "root": api.SCHED_ROOT, "cost": api.SCHED_COST, "dense": api.SCHED_DENSE}[policy]
    gC.fill_with_values(0.0)
    nodes = api.matmult_strassen_sparse_sched(gC, gA, gB, spec[4], 0, pol)
    if policy == "none":
        assert nodes == 0
    if policy in ("root", "dense"):
        assert nodes == 1
    ref = A @ B
    err = np.linalg.norm(gC.to_matrix() - ref) / np.linalg.norm(ref)
    assert err < (1e-14 if policy == "dense" else 1e-6)  # the dense tile screens nothing


def _net_preferring(api, ctx, option, value=-1.0):
    """a network whose prediction is `value` on rows of `option` and 0 on the
    others: hidden unit 0 = relu(one-hot of the option), passed through"""
    net = api.StrassenScheduler(ctx, seed=1)
    IN, H = api.SCHED_FEATURES, 64
    p = np.zeros(net.n_params, np.float32)
    W1, b1 = 0, H * IN
    W2, b2 = b1 + H, b1 + H + H * H
    W3 = b2 + H
    p[W1 + 0 * IN + api.SCHED_NODE_FEATURES + option] = 1.0
    p[W2 + 0 * H + 0] = 1.0
    p[W3 + 0] = value
    net.params = p
    return net


@pytest.mark.parametrize("option", [0, 1, 3])
def test_network_options_reach_the_nodes(api, ctx, option):
    """per-node options from the network: a network that prefers one option
    everywhere makes the root (which covers every node below it) run that
    option -- equal bit for bit to the fixed policy that runs it at the root"""
    spec = (16, 64, 1.0, 2.0, 1e-9, 23)
    A, B, gA, gB, gC = SC.build(spec, ctx)
    net = _net_preferring(api, ctx, option)
    X = api.option_rows(np.zeros(api.SCHED_NODE_FEATURES), range(api.SCHED_OPTIONS))
    yo, _ = mlp.forward(net.params.astype(np.float64), X.astype(np.float64))
    assert np.argmin(yo) == option and yo.min() < 0
    gC.fill_with_values(0.0)
    assert api.matmult_strassen_sparse_sched(gC, gA, gB, spec[4], 0, api.SCHED_MLP, net) == 1
    pol, ms = SC.option_policy(option, spec[0], spec[1])
    gR = api.BlockSparseMatrix(A.shape[0], A.shape[0], 64, 64, 0.0, ctx=ctx)
    gR.fill_with_values(0.0)
    assert api.matmult_strassen_sparse_sched(gR, gA, gB, spec[4], ms, pol) == 1
    assert np.array_equal(gC.to_matrix(), gR.to_matrix())
    # predictions >= 0 everywhere: no node leaves the sparse recursion
    gC.fill_with_values(0.0)
    assert api.matmult_strassen_sparse_sched(gC, gA, gB, spec[4], 0, api.SCHED_MLP,
                                             _net_preferring(api, ctx, option, 1.0)) == 0


@pytest.mark.parametrize("form", ["ozaki", "fp64"])
def test_scheduler_trained_on_every_level(api, ctx, form):
    """Train on timings of the library's own paths on nodes of every level
    (each option of a node against its sparse recursion), evaluate on held-out
    problems against every fixed policy.  The error bound is unchanged: under
    every policy ||C - A B||_F stays within the method's screening bound plus
    the form's arithmetic error.  Times are reported, not asserted (the
    recorded comparison is profiles/strassen_scheduler_gain.md)."""
    fm = api.FORM_OZAKI if form == "ozaki" else api.FORM_FP64
    X, y, meta = SC.collect(SC.problem_specs(1, 8, sizes=(8, 16)), ctx, form=fm, n_digits=4, per_level=1, reps=2)
    levels = {m[1] for m in meta}
    assert len(X) >= 16 and len(levels) >= 3, "training rows from several levels"
    assert {m[2] for m in meta} == set(range(len(SC.OPTIONS))), "every option timed"
    net = api.StrassenScheduler(ctx, seed=9)
    loss = net.train(X, y, epochs=200, batch=32, lr=3e-3, seed=2)
    rows = SC.evaluate(SC.problem_specs(2, 4, sizes=(8, 16)), ctx, net, form=fm, n_digits=4, reps=2)
    print(SC.report(rows, form, len(X), loss))
    arith = 5e-7 if fm == api.FORM_OZAKI else 1e-12  # relative arithmetic error of the form
    for r in rows:
        lim = r["screen_bound"] + arith * r["ref_norm"]
        for name in [n for n in r if isinstance(r[n], dict)]:
            assert r[name]["abs_err"] <= lim, (name, r)
        assert r["regret"] > 0
