"""Edge cases of the mixed form and the batched calls: empty operands, zero
sizes, ragged edge blocks, out-of-range digit counts, unsupported shapes."""
import numpy as np
import pytest

from strassen_gb300 import synth as S

pytestmark = pytest.mark.gpu


def test_mixed_matmult_all_screened(api, ctx):
    a = S.decay_matrix(1, 1, 64, 64, 16, 1.0) * 1e-12
    A = api.BlockSparseMatrix.from_dense(a, 16, 16, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix.from_dense(a, 16, 16, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(64, 64, 16, 16, 0.0, ctx=ctx)
    assert api.matmult(C, A, 0, B, 0, 1.0, form=api.FORM_OZAKI) == 0  # every triple screened out
    assert C.no_of_alloc_blocks() == 0


def test_mixed_matmult_empty_operands(api, ctx):
    A = api.BlockSparseMatrix(40, 24, 8, 8, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix(24, 16, 8, 8, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(40, 16, 8, 8, 0.0, ctx=ctx)
    assert api.matmult(C, A, 0, B, 0, 0.0, form=api.FORM_OZAKI) == 0
    assert not C.to_matrix().any()


@pytest.mark.parametrize("m,k,n,bs", [(77, 53, 29, 16), (130, 70, 45, 24), (65, 65, 65, 32)])
def test_mixed_matmult_ragged(api, ctx, m, k, n, bs):
    a = S.decay_matrix(2, 1, m, k, bs, 2.0)
    b = S.decay_matrix(2, 2, k, n, bs, 2.0)
    A = api.BlockSparseMatrix.from_dense(a, bs, bs, 0.0, ctx=ctx)
    B = api.BlockSparseMatrix.from_dense(b, bs, bs, 0.0, ctx=ctx)
    C64 = api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx)
    Cmx = api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx)
    n64 = api.matmult(C64, A, 0, B, 0, 1e-12)
    nmx = api.matmult(Cmx, A, 0, B, 0, 1e-12, form=api.FORM_OZAKI, n_digits=5)
    assert n64 == nmx and np.array_equal(C64.mask(), Cmx.mask())
    r = C64.to_matrix()
    assert np.linalg.norm(Cmx.to_matrix() - r) <= 1e-9 * np.linalg.norm(r)


def test_mixed_digit_counts_checked(api, ctx):
    a = S.decay_matrix(3, 1, 32, 32, 16, 1.0)
    A = api.BlockSparseMatrix.from_dense(a, 16, 16, 0.0, ctx=ctx)
    C = api.BlockSparseMatrix(32, 32, 16, 16, 0.0, ctx=ctx)
    for nd in (1, 9):
        with pytest.raises(api.BsgError) as e:
            api.matmult(C, A, 0, A, 0, 0.0, form=api.FORM_OZAKI, n_digits=nd)
        assert e.value.code == 1
    a64 = S.decay_matrix(3, 2, 128, 128, 64, 1.0)
    A64 = api.BlockSparseMatrix.from_dense(a64, 64, 64, 0.0, ctx=ctx)
    C64 = api.BlockSparseMatrix(128, 128, 64, 64, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError) as e:  # 8 digits of 64-blocks do not fit two pipeline stages
        api.matmult(C64, A64, 0, A64, 0, 0.0, form=api.FORM_OZAKI, n_digits=8)
    assert e.value.code == 6


def test_mixed_3c2c_ragged_and_empty(api, ctx):
    rng = np.random.default_rng(4)
    n_vec2, n_aux, bs = 203, 61, 24  # neither a multiple of the block size
    X = np.asfortranarray(rng.normal(size=(n_vec2, n_aux)))
    V = np.asfortranarray(rng.normal(size=(n_aux, n_aux)))
    b64 = api.transform_3c2c(X, V, bs, 1e-12, ctx=ctx)
    bmx = api.transform_3c2c(X, V, bs, 1e-12, form=api.FORM_OZAKI, n_digits=6, ctx=ctx)
    assert np.linalg.norm(bmx - b64) <= 1e-10 * np.linalg.norm(b64)
    e = api.transform_3c2c(X[:, :0], V[:0, :0], bs, 1e-12, form=api.FORM_OZAKI, ctx=ctx)
    assert e.shape == (n_vec2, 0)


def test_mixed_rik_zero_sizes(api, ctx, h2o):
    d = h2o
    K = api.rik_occ_step(d["ints"][:, :0], d["keys"], d["c"], d["n_bf"], 0, d["n_occ"], 3, 1e-20,
                         form=api.FORM_OZAKI, ctx=ctx)
    assert not K.any()
    K = api.rik_occ_step(d["ints"][:0], d["keys"][:0], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20,
                         form=api.FORM_OZAKI, ctx=ctx)  # no significant pairs: U empty
    assert not K.any()


def test_batched_edges(api, ctx):
    assert api.matmult_batched([], [], [], 1e-10, form=api.FORM_OZAKI) == 0
    A = api.BlockSparseMatrix(32, 32, 16, 16, 0.0, ctx=ctx)  # empty operand in a batch
    a = S.decay_matrix(5, 1, 48, 48, 16, 1.0)
    B2 = api.BlockSparseMatrix.from_dense(a, 16, 16, 0.0, ctx=ctx)
    C1 = api.BlockSparseMatrix(32, 32, 16, 16, 0.0, ctx=ctx)
    C2 = api.BlockSparseMatrix(48, 48, 16, 16, 0.0, ctx=ctx)
    n = api.matmult_batched([C1, C2], [A, B2], [A, B2], 1e-10, form=api.FORM_OZAKI)
    ref = api.BlockSparseMatrix(48, 48, 16, 16, 0.0, ctx=ctx)
    assert n == api.matmult(ref, B2, 0, B2, 0, 1e-10)
    assert C1.no_of_alloc_blocks() == 0
    r = ref.to_matrix()
    assert np.linalg.norm(C2.to_matrix() - r) <= 1e-9 * np.linalg.norm(r)
    bad = api.BlockSparseMatrix(48, 40, 16, 8, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError):
        api.matmult_batched([C1], [bad], [B2], 1e-10, form=api.FORM_OZAKI)
