"""Screened block GEMM on the GPU (FP64 form) vs the oracle and the
reference's golden outputs: results, block masks, norms and the number of
surviving block products bit-identical (blocksparsematrix.hpp:293-414)."""
import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits
from tests.test_oracle import _mm_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("i", range(6))
def test_matmult_golden(api, ctx, ref_cases, i):
    p = _mm_inputs(ref_cases, i)
    bs = p["bs"]
    A = api.BlockSparseMatrix.from_dense(p["A"], bs, bs, 1e-12, ctx=ctx)
    B = api.BlockSparseMatrix.from_dense(p["B"], bs, bs, 1e-12, ctx=ctx)
    C = api.BlockSparseMatrix(p["m"], p["n"], bs, bs, 1e-3, ctx=ctx)
    if p["c_mode"] == 1:
        C.fill_with_values(0.0)
    if p["c_mode"] == 2:
        C.copy_from_input_matrix(p["Cin"])
    api.matmult(C, A, p["tA"], B, p["tB"], p["thresh"], p["alpha"], p["beta"])
    assert same_bits(C.to_matrix(), ref_cases[f"mm{i}_out"])
    assert np.array_equal(C.mask(), ref_cases[f"mm{i}_mask"])
    assert same_bits(C.norms(), ref_cases[f"mm{i}_norms"])


CASES = [
    # m, k, n, bs, tA, tB, alpha, beta, thresh, L
    (64, 64, 64, 8, 0, 0, 1.0, 0.0, 1e-8, 1.0),
    (100, 77, 53, 9, 1, 0, 1.0, 1.0, 1e-6, 0.7),
    (77, 100, 53, 9, 0, 1, -0.5, 0.0, 1e-6, 0.7),
    (61, 61, 61, 10, 1, 1, 2.0, 3.0, 1e-9, 1.5),
    (256, 256, 256, 64, 0, 0, 1.0, 0.0, 1e-10, 3.0),
    (240, 192, 216, 24, 0, 0, 1.0, 1.0, 1e-10, 0.8),
    (5, 3, 4, 3, 0, 0, 1.0, 0.0, 0.0, 1.0),
    (128, 96, 160, 32, 1, 0, 1.0, 0.0, 1e-5, 0.5),
]


@pytest.mark.parametrize("case", CASES)
def test_matmult_vs_oracle(api, oracle, ctx, case):
    m, k, n, bs, tA, tB, al, be, thr, L = case
    ash = (k, m) if tA else (m, k)
    bsh = (n, k) if tB else (k, n)
    a = S.decay_matrix(21, 1, ash[0], ash[1], bs, L)
    b = S.decay_matrix(21, 2, bsh[0], bsh[1], bs, L)
    c0 = S.decay_matrix(21, 3, m, n, bs, L)
    gA = api.BlockSparseMatrix.from_dense(a, bs, bs, 1e-9, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(b, bs, bs, 1e-9, ctx=ctx)
    gC = api.BlockSparseMatrix.from_dense(c0, bs, bs, 1e-4, ctx=ctx)
    oA = oracle.OBsm(*a.shape, bs, bs, 1e-9, a)
    oB = oracle.OBsm(*b.shape, bs, bs, 1e-9, b)
    oC = oracle.OBsm(m, n, bs, bs, 1e-4, c0)
    ng = api.matmult(gC, gA, tA, gB, tB, thr, al, be)
    no = oracle.matmult(oC, oA, tA, oB, tB, thr, al, be)
    assert ng == no
    assert same_bits(gC.to_matrix(), oC.to_dense())
    assert np.array_equal(gC.mask(), oC.mask())
    assert same_bits(gC.norms(), oC.norms())


def test_matmult_screened_vs_dense(api, ctx):
    """config-1 shape property: thresh 1e-10 screens nothing, result equals
    the dense product to FP64 rounding"""
    n, bs = 512, 64
    a = S.decay_matrix(1, 0, n, n, bs, 6.0)
    b = S.decay_matrix(1, 1, n, n, bs, 6.0)
    A = api.BlockSparseMatrix.from_dense(a, bs, bs, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix.from_dense(b, bs, bs, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    nsig = api.matmult(C, A, 0, B, 0, 1e-10, 1.0, 0.0)
    assert nsig == (n // bs) ** 3
    ref = a @ b
    assert np.linalg.norm(C.to_matrix() - ref) / np.linalg.norm(ref) < 1e-14


def test_matmult_errors(api, ctx):
    A = api.BlockSparseMatrix(8, 6, 2, 2, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix(8, 6, 2, 2, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(8, 6, 2, 2, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError):
        api.matmult(C, A, 0, B, 0, 0.0)
    A2 = api.BlockSparseMatrix(8, 6, 2, 3, 0.0, ctx=ctx)
    B2 = api.BlockSparseMatrix(6, 6, 2, 2, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError):
        api.matmult(C, A2, 0, B2, 0, 0.0)


def test_matmult_empty(api, ctx):
    A = api.BlockSparseMatrix(16, 16, 4, 4, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix(16, 16, 4, 4, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(16, 16, 4, 4, 0.0, ctx=ctx)
    assert api.matmult(C, A, 0, B, 0, 0.0) == 0
    assert C.no_of_alloc_blocks() == 0


def test_tensormult(api, oracle, ctx):
    """contract: C = sum_l A^l B^l; batched: C^l = A B^l -- against the oracle
    matmult chained in the same accumulation order"""
    n, bs, L = 48, 8, 3
    As = [S.decay_matrix(9, l, n, n, bs, 1.0) for l in range(L)]
    Bs = [S.decay_matrix(9, 10 + l, n, n, bs, 1.0) for l in range(L)]
    gA = [api.BlockSparseMatrix.from_dense(a, bs, bs, 1e-6, ctx=ctx) for a in As]
    gB = [api.BlockSparseMatrix.from_dense(b, bs, bs, 1e-6, ctx=ctx) for b in Bs]
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    api.tensormult_contract(gC, gA, 0, gB, 0, 1e-5)
    oC = oracle.OBsm(n, n, bs, bs, 0.0)
    for l in range(L):  # beta 0 once, then accumulate slice by slice
        oracle.matmult(oC, oracle.OBsm(n, n, bs, bs, 1e-6, As[l]), 0, oracle.OBsm(n, n, bs, bs, 1e-6, Bs[l]), 0, 1e-5,
                       1.0, 0.0 if l == 0 else 1.0)
    assert same_bits(gC.to_matrix(), oC.to_dense())
    gCs = [api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx) for _ in range(L)]
    api.tensormult_batched(gCs, gA[0], 1, gB, 0, 1e-5)
    for l in range(L):
        o = oracle.OBsm(n, n, bs, bs, 0.0)
        oracle.matmult(o, oracle.OBsm(n, n, bs, bs, 1e-6, As[0]), 1, oracle.OBsm(n, n, bs, bs, 1e-6, Bs[l]), 0, 1e-5)
        assert same_bits(gCs[l].to_matrix(), o.to_dense())
