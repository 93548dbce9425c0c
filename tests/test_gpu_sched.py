"""Learned Strassen scheduler: the device forward / backward kernels against
the CPU oracle, training, node features, and the measured gain of the trained
network over the reference's cost model on held-out problems."""
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


@pytest.mark.parametrize("policy", ["none", "root", "cost"])
def test_policies_give_the_product(api, ctx, policy):
    spec = (16, 64, 0.5, 2.0, 1e-9, 21)
    A, B, gA, gB, gC = SC.build(spec, ctx)
    pol = {"none": api.SCHED_NONE, "root": api.SCHED_ROOT, "cost": api.SCHED_COST}[policy]
    gC.fill_with_values(0.0)
    nodes = api.matmult_strassen_sparse_sched(gC, gA, gB, spec[4], 0, pol)
    if policy == "none":
        assert nodes == 0
    if policy == "root":
        assert nodes == 1
    ref = A @ B
    assert np.linalg.norm(gC.to_matrix() - ref) / np.linalg.norm(ref) < 1e-6  # screening error only


@pytest.mark.parametrize("form", ["ozaki", "fp64"])
def test_scheduler_gain_over_cost_model(api, ctx, form):
    """Train on timings of the library's own paths, evaluate on held-out
    problems: time under the network vs under the cost model.  The error bound
    is unchanged: under either policy ||C - A B||_F stays within the method's
    screening bound plus the form's arithmetic error."""
    fm = api.FORM_OZAKI if form == "ozaki" else api.FORM_FP64
    train = SC.problem_specs(1, 28)
    test = SC.problem_specs(2, 10)
    X, y = SC.collect(train, ctx, form=fm, n_digits=4)
    assert len(X) >= 8
    net = api.StrassenScheduler(ctx, seed=9)
    loss = net.train(X, y, epochs=300, batch=16, lr=3e-3, seed=2)
    rows = SC.evaluate(test, ctx, net, form=fm, n_digits=4)
    t_cost = sum(r["cost"]["s"] for r in rows)
    t_mlp = sum(r["mlp"]["s"] for r in rows)
    print(f"scheduler [{form}] train samples {len(X)} loss {loss:.4f}: held-out time cost model {t_cost * 1e3:.1f} ms, "
          f"network {t_mlp * 1e3:.1f} ms, gain x{t_cost / t_mlp:.2f}")
    for r in rows:
        print("  ", r["spec"][:5], "bound %.1e" % (r["screen_bound"] / r["ref_norm"]),
              "cost %.2f ms (%d nodes, err %.1e)" % (r["cost"]["s"] * 1e3, r["cost"]["nodes"], r["cost"]["rel_err"]),
              "mlp %.2f ms (%d nodes, err %.1e)" % (r["mlp"]["s"] * 1e3, r["mlp"]["nodes"], r["mlp"]["rel_err"]))
    arith = 5e-7 if fm == api.FORM_OZAKI else 1e-12  # relative arithmetic error of the form
    for r in rows:
        lim = r["screen_bound"] + arith * r["ref_norm"]
        assert r["mlp"]["abs_err"] <= lim and r["cost"]["abs_err"] <= lim, r
    assert t_mlp <= 1.10 * t_cost  # never materially slower than the method without it
