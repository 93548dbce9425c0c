"""Hybrid Strassen-Winograd / sparse recursion on the GPU (FP64 form): decision
trees, per-level flop counts and results bit-identical to the reference."""
import hashlib

import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits
from tests.test_oracle import _st_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("i", range(5))
def test_strassen_golden(api, ctx, ref_cases, i):
    n, bs, thr, ms, A, B = _st_inputs(ref_cases, i)
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    levels, flops = api.matmult_strassen_dryrun(gA, gB, thr * bs ** 3)
    tree = np.concatenate(levels).astype(np.uint8) if levels else np.zeros(0, np.uint8)
    assert np.array_equal(tree, ref_cases[f"st{i}_tree"])
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    gC.fill_with_values(0.0)
    api.matmult_strassen_sparse(gC, gA, 0, gB, 0, thr, 1.0, 0.0, ms)
    out = np.asfortranarray(gC.to_matrix())
    assert hashlib.sha256(out.tobytes(order="F")).hexdigest() == str(ref_cases[f"st{i}_sha256"])


@pytest.mark.parametrize("n,bs,L,core,thr,ms", [(512, 32, 1.0, 256, 1e-7, 0), (384, 32, 2.0, 128, 1e-4, 64),
                                                  (640, 32, 1.5, 320, 1e-6, 64), (1024, 16, 3.0, 512, 1e-8, 128),
                                                  (96, 8, 2.0, 0, 0.0, 8)])
def test_strassen_vs_oracle(api, oracle, ctx, n, bs, L, core, thr, ms):
    A = S.decay_matrix(4, 1, n, n, bs, L, core=core)
    B = S.decay_matrix(4, 2, n, n, bs, L, core=core)
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    oA = oracle.OBsm(n, n, bs, bs, 0.0, A)
    oB = oracle.OBsm(n, n, bs, bs, 0.0, B)
    lg, fg = api.matmult_strassen_dryrun(gA, gB, thr * bs ** 3)
    lo, fo = oracle.strassen_dryrun(oA, oB, thr * bs ** 3)
    assert len(lg) == len(lo) and all(np.array_equal(a.astype(np.uint8), b) for a, b in zip(lg, lo))
    assert np.array_equal(fg, fo)
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    gC.fill_with_values(0.0)
    oC = oracle.OBsm(n, n, bs, bs, 0.0)
    oC.fill(0.0)
    api.matmult_strassen_sparse(gC, gA, 0, gB, 0, thr, 1.0, 0.0, ms)
    oracle.matmult_strassen_sparse(oC, oA, oB, thr, ms)
    assert same_bits(gC.to_matrix(), oC.to_dense())


def test_strassen_preconditions(api, ctx):
    n, bs = 256, 32
    A = S.decay_matrix(4, 3, n, n, bs, 50.0)
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)  # not pre-filled
    with pytest.raises(api.BsgError) as e:
        api.matmult_strassen_sparse(gC, gA, 0, gB, 0, 0.0, 1.0, 0.0, 64)
    assert e.value.code == 2
    with pytest.raises(api.BsgError):
        api.matmult_strassen_sparse(gC, gA, 1, gB, 0, 0.0, 1.0, 0.0, 64)
    with pytest.raises(api.BsgError):
        api.matmult_strassen_sparse(gC, gA, 0, gB, 0, 0.0, 2.0, 0.0, 64)


@pytest.mark.parametrize("n,bs,L,core,thr,ms,nd", [(512, 32, 1.0, 256, 1e-7, 128, 4), (1024, 64, 6.0, 512, 1e-9, 256, 4),
                                                   (768, 24, 2.0, 384, 1e-8, 96, 5), (2048, 64, 6.0, 2048, 1e-10, 1024, 4)])
def test_strassen_mixed_form(api, ctx, n, bs, L, core, thr, ms, nd):
    """Mixed form: Winograd leaves as bf16 digit products on the tensor cores,
    pre/post sums and the screened sparse part in FP64.  Same decision tree
    and the same C block structure as the FP64 form; relative Frobenius error
    within the digit bound."""
    A = S.decay_matrix(5, 1, n, n, bs, L, core=core)
    B = S.decay_matrix(5, 2, n, n, bs, L, core=core)
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    C64 = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    Cmx = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    C64.fill_with_values(0.0)
    Cmx.fill_with_values(0.0)
    api.matmult_strassen_sparse(C64, gA, 0, gB, 0, thr, 1.0, 0.0, ms)
    api.matmult_strassen_sparse(Cmx, gA, 0, gB, 0, thr, 1.0, 0.0, ms, form=api.FORM_OZAKI, n_digits=nd)
    assert np.array_equal(C64.mask(), Cmx.mask())
    r64, rmx = C64.to_matrix(), Cmx.to_matrix()
    err = np.linalg.norm(rmx - r64) / np.linalg.norm(r64)
    print("strassen mixed form", n, bs, nd, err)
    assert err < {4: 1e-7, 5: 1e-9}[nd], err
