"""Batched screened products (one persistent tensor-core launch over every
block-size group, per-group autotuning, CUDA-graph plans) against the
per-product FP64 matmult."""
import numpy as np
import pytest

from strassen_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _batch(api, ctx, seed, n, sizes=(96, 128, 192, 256, 320), bss=(16, 32, 48, 64), cycle=False):
    """n seeded products; block sizes drawn from bss (cycle: bss in turn)"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        bs = int(bss[i % len(bss)]) if cycle else int(rng.choice(bss))
        m, k, nn = (int(rng.choice(sizes)) // bs * bs or bs for _ in range(3))
        dens = float(rng.uniform(0.05, 0.6))
        a = S.block_mask_matrix(seed * 100 + i, 1, m, k, bs, dens)
        b = S.block_mask_matrix(seed * 100 + i, 2, k, nn, bs, dens)
        gA = api.BlockSparseMatrix.from_dense(a, bs, bs, 1e-12, ctx=ctx)
        gB = api.BlockSparseMatrix.from_dense(b, bs, bs, 1e-12, ctx=ctx)
        out.append((bs, m, nn, gA, gB))
    return out


def _outs(api, ctx, batch):
    return [api.BlockSparseMatrix(m, nn, bs, bs, 0.0, ctx=ctx) for bs, m, nn, _, _ in batch]


def test_batched_mixed_matches_fp64(api, ctx):
    batch = _batch(api, ctx, 3, 14)
    C64, Cmx = _outs(api, ctx, batch), _outs(api, ctx, batch)
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    thr = 1e-9
    n64 = sum(api.matmult(c, a, 0, b, 0, thr, 1.0, 0.0) for c, a, b in zip(C64, As, Bs))
    nmx = api.matmult_batched(Cmx, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)
    assert n64 == nmx
    for (bs, *_), c64, cmx in zip(batch, C64, Cmx):
        assert np.array_equal(c64.mask(), cmx.mask())
        r64, rmx = c64.to_matrix(), cmx.to_matrix()
        err = np.linalg.norm(rmx - r64) / max(np.linalg.norm(r64), 1e-300)
        assert err < (1e-7 if bs == 64 else 1e-9), (bs, err)
    tuned = ctx.autotune_entries()
    assert len(tuned) >= 1  # one entry per block-size group shape
    for (mp, kp, np_, nd), (R, S_) in tuned.items():
        assert 1 <= R <= 128 // mp and S_ in (0, 2)


def test_batched_one_launch_over_block_sizes(api, ctx):
    """A batch of four block sizes runs as ONE persistent tensor-core launch,
    each tile in its group's geometry (once the autotuner has cached its
    choices: its trial launches run group by group), and every product stays
    within the form's bound of the per-product FP64 matmult with its mask."""
    batch = _batch(api, ctx, 11, 12)
    assert len({b[0] for b in batch}) >= 3
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    C64, Cmx = _outs(api, ctx, batch), _outs(api, ctx, batch)
    thr = 1e-9
    n64 = sum(api.matmult(c, a, 0, b, 0, thr, 1.0, 0.0) for c, a, b in zip(C64, As, Bs))
    api.matmult_batched(Cmx, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)  # tunes the group shapes
    for c in Cmx:
        c.scale(0.0)
    ctx.set_timing(True)
    try:
        nmx = api.matmult_batched(Cmx, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)
        launches = ctx.gemm_timing()[0]
    finally:
        ctx.set_timing(False)
    assert launches == 1
    assert n64 == nmx
    for (bs, *_), c64, cmx in zip(batch, C64, Cmx):
        assert np.array_equal(c64.mask(), cmx.mask())
        r64, rmx = c64.to_matrix(), cmx.to_matrix()
        err = np.linalg.norm(rmx - r64) / max(np.linalg.norm(r64), 1e-300)
        assert err < (1e-7 if bs == 64 else 1e-9), (bs, err)


@pytest.mark.parametrize("bss", [(8, 24, 40, 56), (8, 12, 16, 20, 24, 28, 32, 40, 48)])
def test_batched_geometries_in_one_launch(api, ctx, bss):
    """Geometries that differ in more than the tile width share a launch:
    step pairs (block sizes 8, 24 and 40: k = 8 mod 16), 8-row blocks whose
    slots hold only 64 of the MMA's 128 rows, 56-wide blocks at 4 digits next
    to 5-digit ones; more than eight block-size groups take one launch per
    eight groups.  Every product keeps the FP64 form's mask and bound."""
    batch = _batch(api, ctx, 13, 3 * len(bss), sizes=(96, 160, 224), bss=bss, cycle=True)
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    C64, Cmx = _outs(api, ctx, batch), _outs(api, ctx, batch)
    thr = 1e-9
    n64 = sum(api.matmult(c, a, 0, b, 0, thr, 1.0, 0.0) for c, a, b in zip(C64, As, Bs))
    api.matmult_batched(Cmx, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)  # tunes the group shapes
    groups = len({b[0] for b in batch})
    assert groups == len(bss)
    ctx.set_timing(True)
    try:
        nmx = api.matmult_batched(Cmx, As, Bs, thr, 1.0, 0.0, form=api.FORM_OZAKI)
        launches = ctx.gemm_timing()[0]
    finally:
        ctx.set_timing(False)
    assert launches == -(-groups // 8)
    assert n64 == nmx
    for (bs, *_), c64, cmx in zip(batch, C64, Cmx):
        assert np.array_equal(c64.mask(), cmx.mask())
        r64, rmx = c64.to_matrix(), cmx.to_matrix()
        err = np.linalg.norm(rmx - r64) / max(np.linalg.norm(r64), 1e-300)
        assert err < (1e-7 if bs >= 56 else 1e-9), (bs, err)


def test_batched_fp64_is_bit_exact(api, ctx):
    batch = _batch(api, ctx, 5, 6)
    C1, C2 = _outs(api, ctx, batch), _outs(api, ctx, batch)
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    for c, a, b in zip(C1, As, Bs):
        api.matmult(c, a, 0, b, 0, 1e-8, 0.5, 0.0)
    api.matmult_batched(C2, As, Bs, 1e-8, 0.5, 0.0, form=api.FORM_FP64)
    for c1, c2 in zip(C1, C2):
        assert np.array_equal(c1.mask(), c2.mask())
        assert np.array_equal(c1.to_matrix().view(np.uint64), c2.to_matrix().view(np.uint64))


def test_batched_beta_accumulates(api, ctx):
    batch = _batch(api, ctx, 7, 4, bss=(32,))
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    C1 = _outs(api, ctx, batch)
    api.matmult_batched(C1, As, Bs, 1e-10, 1.0, 0.0, form=api.FORM_OZAKI)
    first = [c.to_matrix() for c in C1]
    api.matmult_batched(C1, As, Bs, 1e-10, 1.0, 1.0, form=api.FORM_OZAKI)  # C += A B
    for f, c in zip(first, C1):
        assert np.allclose(c.to_matrix(), 2 * f, rtol=1e-9, atol=1e-12 * np.abs(f).max())


def test_batch_plan_replays(api, ctx):
    batch = _batch(api, ctx, 9, 8)
    As = [b[3] for b in batch]
    Bs = [b[4] for b in batch]
    Cref, Cp = _outs(api, ctx, batch), _outs(api, ctx, batch)
    api.matmult_batched(Cref, As, Bs, 1e-9, 1.0, 0.0, form=api.FORM_OZAKI)
    plan = api.BatchPlan(Cp, As, Bs, 1e-9)
    first = [c.to_matrix() for c in Cp]
    for c in Cp:
        c.scale(0.0)  # values gone, blocks kept (a plan needs C's block structure unchanged)
    plan.run()
    plan.run()
    for r, f, c in zip(Cref, first, Cp):
        assert np.array_equal(r.mask(), c.mask())
        assert np.array_equal(f.view(np.uint64), c.to_matrix().view(np.uint64))  # a replay overwrites (beta 0)
        rr = r.to_matrix()
        assert np.linalg.norm(c.to_matrix() - rr) <= 1e-7 * max(np.linalg.norm(rr), 1e-300)
