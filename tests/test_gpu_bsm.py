"""BlockSparseMatrix container operations on the GPU vs the oracle: values,
block masks and cached norms bit-identical (blocksparsematrix.hpp:35-261)."""
import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits

pytestmark = pytest.mark.gpu


def pair(api, oracle, ctx, a, bs, thresh):
    g = api.BlockSparseMatrix.from_dense(a, bs[0], bs[1], thresh, ctx=ctx)
    o = oracle.OBsm(a.shape[0], a.shape[1], bs[0], bs[1], thresh, a)
    return g, o


def same(g, o):
    return same_bits(g.to_matrix(), o.to_dense()) and np.array_equal(g.mask(), o.mask()) and same_bits(g.norms(), o.norms())


@pytest.mark.parametrize("shape,bs,thr", [((40, 40), (6, 6), 1e-3), ((37, 53), (5, 8), 1e-2), ((64, 64), (16, 16), 0.0),
                                          ((3, 7), (4, 4), 1e-20), ((96, 200), (24, 24), 1e-4)])
def test_copy_from_dense_screen(api, oracle, ctx, shape, bs, thr):
    a = S.decay_matrix(1, 0, shape[0], shape[1], bs[0], 1.2)
    g, o = pair(api, oracle, ctx, a, bs, thr)
    assert same(g, o)
    assert g.no_of_alloc_blocks() == o.no_of_alloc_blocks()
    assert g.frobenius_norm() == o.frobenius_norm()


@pytest.mark.parametrize("op", ["add", "sub", "add_transpose", "scale", "recompress", "calc_norms", "fill", "zero",
                                "assign"])
def test_container_ops(api, oracle, ctx, op):
    n, bs, thr = 46, (6, 6), 1e-3
    L_ = S.decay_matrix(2, 1, n, n, bs[0], 2.0)
    R_ = S.decay_matrix(2, 2, n, n, bs[0], 2.0)
    gl, ol = pair(api, oracle, ctx, L_, bs, thr)
    gr, orr = pair(api, oracle, ctx, R_, bs, thr)
    if op == "add":
        gl += gr
        ol.add(orr)
    elif op == "sub":
        gl -= gr
        ol.sub(orr)
    elif op == "add_transpose":
        gl.add_transpose(gr)
        ol.add_transpose(orr)
    elif op == "scale":
        gl *= -0.75
        ol.scale(-0.75)
    elif op == "recompress":
        gl.scale(1e-2)
        ol.scale(1e-2)
        gl.recompress()
        ol.recompress()
    elif op == "calc_norms":
        gl.scale(3.0)
        ol.scale(3.0)
        gl.calc_frobenius_norms()
        ol.calc_norms()
    elif op == "fill":
        gl.fill_with_values(0.5)
        ol.fill(0.5)
    elif op == "zero":
        gl.zero()
        ol.zero()
    elif op == "assign":
        gl.assign(gr)
        ol.copy_from(orr)
    assert same(gl, ol)
    assert gl.frobenius_norm() == ol.frobenius_norm()


def test_dot(api, oracle, ctx):
    a = S.decay_matrix(3, 1, 50, 50, 7, 1.0)
    b = S.decay_matrix(3, 2, 50, 50, 7, 1.0)
    ga, oa = pair(api, oracle, ctx, a, (7, 7), 1e-3)
    gb, ob = pair(api, oracle, ctx, b, (7, 7), 1e-3)
    for thr in (0.0, 1e-2):
        assert api.dot(ga, gb, thr) == oracle.dot(oa, ob, thr)


def test_shared_pool(api, ctx):
    pool = api.BlockMemoryPool(16, ctx=ctx)
    a = api.BlockSparseMatrix(12, 12, 4, 4, 0.0, pool=pool)
    b = api.BlockSparseMatrix(8, 8, 4, 4, 0.0, pool=pool)
    a.fill_with_values(1.0)
    b.fill_with_values(2.0)
    st = pool.stats()
    assert st["blocks_total"] - st["blocks_free"] == 9 + 4
    del a
    st2 = pool.stats()
    assert st2["blocks_total"] - st2["blocks_free"] == 4
    assert np.all(b.to_matrix() == 2.0)


def test_dimension_mismatch_is_an_error(api, ctx):
    a = api.BlockSparseMatrix(8, 8, 4, 4, 0.0, ctx=ctx)
    b = api.BlockSparseMatrix(8, 12, 4, 4, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError):
        a += b
    with pytest.raises(api.BsgError):
        a.add_transpose(b)
