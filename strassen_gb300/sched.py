"""Training data, training and evaluation of the learned Strassen scheduler.

The scheduler (a 2 x 64 MLP, `api.StrassenScheduler`) predicts, for a node of
the Strassen decision tree, y = log(t_strassen / t_sparse) from 25 node
features (`api.strassen_root_features`).  Its training data are timings the
library takes of its own paths: for a square product whose root node may run
Strassen, the time with Strassen at the root (policy ROOT) against the time
without any Strassen node (policy NONE).  At run time (policy MLP) every
eligible node of the tree is scheduled by the network, the reference's cost
model covering the levels with more than 65536 nodes.
"""
from __future__ import annotations

import time

import numpy as np

from . import api
from . import synth as S


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


def build(spec, ctx):
    nb, bs, core, L, thr, sd = spec
    n = nb * bs
    A = S.decay_matrix(sd, 1, n, n, bs, L, core=int(core * n))
    B = S.decay_matrix(sd, 2, n, n, bs, L, core=int(core * n))
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    return A, B, gA, gB, gC


def run(gC, gA, gB, thr, min_size, policy, sched=None, form=api.FORM_FP64, n_digits=4, reps=3):
    """median wall time (s) of the synchronous call and the number of Strassen nodes"""
    ts, nodes = [], 0
    for _ in range(reps):
        gC.fill_with_values(0.0)
        t0 = time.perf_counter()
        nodes = api.matmult_strassen_sparse_sched(gC, gA, gB, thr, min_size, policy, sched, form, n_digits)
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), nodes


def collect(specs, ctx, form=api.FORM_FP64, n_digits=4, min_size=0, reps=3):
    """features X and labels y = log(t_root / t_none) of the problems whose
    root may run Strassen"""
    X, y = [], []
    for spec in specs:
        _, _, gA, gB, gC = build(spec, ctx)
        thr = spec[4]
        gC.fill_with_values(0.0)
        f, ok = api.strassen_root_features(gC, gA, gB, thr)
        if not ok:
            continue
        run(gC, gA, gB, thr, min_size, api.SCHED_NONE, form=form, n_digits=n_digits, reps=1)  # warm-up
        t_root, _ = run(gC, gA, gB, thr, min_size, api.SCHED_ROOT, form=form, n_digits=n_digits, reps=reps)
        t_none, _ = run(gC, gA, gB, thr, min_size, api.SCHED_NONE, form=form, n_digits=n_digits, reps=reps)
        X.append(f)
        y.append(np.log(t_root / t_none))
    return np.array(X, np.float32).reshape(-1, api.SCHED_FEATURES), np.array(y, np.float32)


def screening_bound(A, B, bs, thresh):
    """the method's screening error bound for C = A B:
    ||C - A B||_F <= sum over dropped block triples of ||A_ik|| ||B_kj||
    (a triple is dropped when ||A_ik|| ||B_kj|| < thresh bs^3)"""
    nb = A.shape[0] // bs
    an = np.linalg.norm(A.reshape(nb, bs, nb, bs), axis=(1, 3))  # an[i, k]
    bn = np.linalg.norm(B.reshape(nb, bs, nb, bs), axis=(1, 3))  # bn[k, j]
    prod = an[:, :, None] * bn[None, :, :]  # [i, k, j]
    return float(prod[prod < thresh * bs ** 3].sum())


def evaluate(specs, ctx, sched, form=api.FORM_FP64, n_digits=4, min_size=0, reps=3):
    """per problem: time, absolute error against the exact product and the
    screening bound, under the cost model and under the network"""
    rows = []
    for spec in specs:
        A, B, gA, gB, gC = build(spec, ctx)
        nb, bs, thr = spec[0], spec[1], spec[4]
        ref = A @ B
        row = {"spec": spec, "ref_norm": float(np.linalg.norm(ref)), "screen_bound": screening_bound(A, B, bs, thr)}
        for name, pol in (("cost", api.SCHED_COST), ("mlp", api.SCHED_MLP)):
            run(gC, gA, gB, thr, min_size, pol, sched, form, n_digits, reps=1)
            t, nodes = run(gC, gA, gB, thr, min_size, pol, sched, form, n_digits, reps=reps)
            err = float(np.linalg.norm(gC.to_matrix() - ref))
            row[name] = {"s": t, "nodes": nodes, "abs_err": err, "rel_err": err / row["ref_norm"]}
        rows.append(row)
    return rows
