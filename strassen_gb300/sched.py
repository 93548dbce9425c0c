"""Training data, training and evaluation of the learned Strassen scheduler.

The scheduler (a 2 x 64 MLP, `api.StrassenScheduler`) scores, for a node of
the hybrid recursion's decision tree (a quadrant product, strassen.hpp:
418-508), each option against the screened sparse recursion: y =
log(t_option / t_sparse) for Strassen-Winograd of depth 1, 2 or 3 at the node
and for the node's product as one dense tile.  Its inputs are the node's 25
features (`api.strassen_root_features`) and the option's one-hot.

Training data are timings the library takes of its own paths on nodes of
every level: a node of level L of a training problem is cut out as a problem
of its own (its 2^(L+1) x 2^(L+1) blocks of A and B), whose root is then that
node, and timed with the sparse recursion only (policy NONE), with Strassen
at the root recursing to the option's depth (policy ROOT with the matching
min_size_for_strassen) and as a dense tile (policy DENSE).  At run time
(policy MLP) every eligible node takes the option the network predicts
fastest where it beats the sparse recursion; the reference's cost model
covers the levels with more than 65536 nodes.
"""
from __future__ import annotations

import time

import numpy as np

from . import api
from . import synth as S

OPTIONS = ("Strassen depth 1", "Strassen depth 2", "Strassen depth 3", "dense tile")


def problem_specs(seed, n, sizes=(8, 16, 32), bs=64):
    """seeded mix of problem structures: (nb, bs, dense core fraction, decay
    length, threshold, seed)"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nb = int(rng.choice(sizes))
        core = float(rng.choice([0.0, 0.25, 0.5, 1.0]))
        L = float(rng.choice([0.5, 1.0, 3.0, 10.0]))
        thr = float(rng.choice([1e-12, 1e-8, 1e-5, 1e-3]))
        out.append((nb, bs, core, L, thr, int(seed * 1000 + i)))
    return out


def matrices(spec):
    nb, bs, core, L, thr, sd = spec
    n = nb * bs
    return (S.decay_matrix(sd, 1, n, n, bs, L, core=int(core * n)),
            S.decay_matrix(sd, 2, n, n, bs, L, core=int(core * n)))


def operands(A, B, bs, ctx):
    n = A.shape[0]
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    return gA, gB, gC


def build(spec, ctx):
    A, B = matrices(spec)
    return (A, B) + operands(A, B, spec[1], ctx)


def run(gC, gA, gB, thr, min_size, policy, sched=None, form=api.FORM_FP64, n_digits=4, reps=3):
    """median wall time (s) of the synchronous call and the number of nodes
    that ran Strassen or a dense tile"""
    ts, nodes = [], 0
    for _ in range(reps):
        gC.fill_with_values(0.0)
        t0 = time.perf_counter()
        nodes = api.matmult_strassen_sparse_sched(gC, gA, gB, thr, min_size, policy, sched, form, n_digits)
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), nodes


def option_policy(opt, nb, bs):
    """(policy, min_size_for_strassen) that runs option `opt` at the root of
    an nb x nb block problem: Strassen recursing while the grid side exceeds
    (nb / 2) / 2^(depth - 1), or the dense tile"""
    if opt == len(OPTIONS) - 1:
        return api.SCHED_DENSE, 0
    return api.SCHED_ROOT, max(1, (nb // 2) >> opt) * bs


def option_valid(opt, level):
    """depth t needs 2^(t-1) to divide the node's half side 2^level"""
    return opt == len(OPTIONS) - 1 or opt <= level


def collect(specs, ctx, form=api.FORM_FP64, n_digits=4, per_level=2, reps=3, seed=0):
    """Training rows (node features + option one-hot), labels
    y = log(t_option / t_sparse) and (spec, level, option) per row, from up
    to `per_level` nodes of every level of every problem, each cut out and
    timed as a problem of its own."""
    rng = np.random.default_rng(seed)
    X, y, meta = [], [], []
    for spec in specs:
        A, B = matrices(spec)
        nb, bs, thr = spec[0], spec[1], spec[4]
        level = 0
        while (2 << level) <= nb:
            sb = 2 << level
            ns = nb // sb
            picks = {(int(rng.integers(ns)), int(rng.integers(ns)), int(rng.integers(ns))) for _ in range(per_level)}
            for si, sj, sk in sorted(picks):
                rs, ks, js = (slice(x * sb * bs, (x + 1) * sb * bs) for x in (si, sk, sj))
                gA, gB, gC = operands(np.asfortranarray(A[rs, ks]), np.asfortranarray(B[ks, js]), bs, ctx)
                gC.fill_with_values(0.0)
                f, ok = api.strassen_root_features(gC, gA, gB, thr)
                if not ok:
                    continue
                run(gC, gA, gB, thr, 0, api.SCHED_NONE, form=form, n_digits=n_digits, reps=1)  # warm-up
                t_none, _ = run(gC, gA, gB, thr, 0, api.SCHED_NONE, form=form, n_digits=n_digits, reps=reps)
                for opt in range(len(OPTIONS)):
                    if not option_valid(opt, level):
                        continue
                    pol, ms = option_policy(opt, sb, bs)
                    t_opt, _ = run(gC, gA, gB, thr, ms, pol, form=form, n_digits=n_digits, reps=reps)
                    X.append(api.option_rows(f, [opt])[0])
                    y.append(np.log(t_opt / t_none))
                    meta.append((spec, level, opt))
            level += 1
    return np.array(X, np.float32).reshape(-1, api.SCHED_FEATURES), np.array(y, np.float32), meta


def screening_bound(A, B, bs, thresh):
    """the method's screening error bound for C = A B:
    ||C - A B||_F <= sum over dropped block triples of ||A_ik|| ||B_kj||
    (a triple is dropped when ||A_ik|| ||B_kj|| < thresh bs^3)"""
    nb = A.shape[0] // bs
    an = np.linalg.norm(A.reshape(nb, bs, nb, bs), axis=(1, 3))  # an[i, k]
    bn = np.linalg.norm(B.reshape(nb, bs, nb, bs), axis=(1, 3))  # bn[k, j]
    prod = an[:, :, None] * bn[None, :, :]  # [i, k, j]
    return float(prod[prod < thresh * bs ** 3].sum())


def fixed_policies(nb, bs):
    """the per-problem fixed choices the network is judged against: the
    reference's cost model, no Strassen, Strassen at the root of each depth,
    the root as a dense tile"""
    out = [("cost", api.SCHED_COST, 0), ("none", api.SCHED_NONE, 0)]
    for t in range(1, 4):
        if (nb // 2) >> (t - 1) >= 1 and (nb // 2) % (1 << (t - 1)) == 0:
            out.append((f"root_depth{t}", api.SCHED_ROOT, max(1, (nb // 2) >> (t - 1)) * bs))
    out.append(("dense", api.SCHED_DENSE, 0))
    return out


def evaluate(specs, ctx, sched, form=api.FORM_FP64, n_digits=4, reps=3):
    """Per problem: time, node count and error (against the exact product and
    the screening bound) of every fixed policy and of the network; the
    network's regret = its time / the best fixed policy's time."""
    rows = []
    for spec in specs:
        A, B, gA, gB, gC = build(spec, ctx)
        nb, bs, thr = spec[0], spec[1], spec[4]
        ref = A @ B
        row = {"spec": spec, "ref_norm": float(np.linalg.norm(ref)), "screen_bound": screening_bound(A, B, bs, thr)}
        pols = fixed_policies(nb, bs) + [("mlp", api.SCHED_MLP, 0)]
        for name, pol, ms in pols:
            run(gC, gA, gB, thr, ms, pol, sched, form, n_digits, reps=1)
            t, nodes = run(gC, gA, gB, thr, ms, pol, sched, form, n_digits, reps=reps)
            err = float(np.linalg.norm(gC.to_matrix() - ref))
            row[name] = {"s": t, "nodes": nodes, "abs_err": err, "rel_err": err / row["ref_norm"]}
        fixed = [n for n, _, _ in pols if n != "mlp"]
        best = min(fixed, key=lambda n: row[n]["s"])
        row["best_fixed"] = best
        row["regret"] = row["mlp"]["s"] / row[best]["s"]
        rows.append(row)
    return rows


def report(rows, form_name, n_train, loss):
    """markdown summary of an evaluation"""
    g = float(np.exp(np.mean([np.log(r["regret"]) for r in rows])))
    tot = {k: sum(r[k]["s"] for r in rows) for k in ("cost", "none", "mlp")}
    best = sum(r[r["best_fixed"]]["s"] for r in rows)
    lines = [f"### {form_name}: {n_train} training rows, final loss {loss:.4f}", "",
             f"Held-out total: network {tot['mlp'] * 1e3:.1f} ms, per-problem best fixed policy {best * 1e3:.1f} ms, "
             f"cost model {tot['cost'] * 1e3:.1f} ms, no Strassen {tot['none'] * 1e3:.1f} ms; geometric-mean regret "
             f"against the best fixed policy x{g:.3f}.", "",
             "| nb, bs, core, L, thresh | bound | best fixed (ms) | network (ms, nodes) | regret | cost model (ms) "
             "| network err |", "|---|---:|---|---|---:|---:|---:|"]
    for r in rows:
        b = r["best_fixed"]
        lines.append(f"| {', '.join(str(x) for x in r['spec'][:5])} | {r['screen_bound'] / r['ref_norm']:.1e} | "
                     f"{b} {r[b]['s'] * 1e3:.2f} | {r['mlp']['s'] * 1e3:.2f}, {r['mlp']['nodes']} | "
                     f"x{r['regret']:.2f} | {r['cost']['s'] * 1e3:.2f} | {r['mlp']['rel_err']:.1e} |")
    return "\n".join(lines)


def main():
    """Train on timings of the library's own paths and report the network on
    held-out problems against every fixed policy (markdown on stdout)."""
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=24)
    ap.add_argument("--test", type=int, default=10)
    ap.add_argument("--forms", default="ozaki,fp64")
    args = ap.parse_args()
    ctx = api.Context(0)
    for fname in args.forms.split(","):
        form = api.FORM_OZAKI if fname == "ozaki" else api.FORM_FP64
        X, y, _ = collect(problem_specs(1, args.train), ctx, form=form, n_digits=4)
        net = api.StrassenScheduler(ctx, seed=9)
        loss = net.train(X, y, epochs=300, batch=32, lr=3e-3, seed=2)
        rows = evaluate(problem_specs(2, args.test), ctx, net, form=form, n_digits=4)
        print(report(rows, "mixed form (bf16 x 4 digits)" if form == api.FORM_OZAKI else "FP64 form", len(X), loss))
        print()


if __name__ == "__main__":
    main()
