"""The Strassen benchmark's shape (main.cpp:28-63): n 2048, block 64, blocks
scaled by exp(-|I-J|/6), inputs stored at threshold 0, products screened at
1e-10, one Winograd level (min_size_for_strassen 1024).  The FP64 form is
checked bit for bit against the compiled reference's results
(tests/golden/config1_golden.npz, made by make_golden.py config1): the
screened matmult's output, block mask, cached norms and surviving-pair count,
the dry-run decision tree, and matmult_strassen_sparse's output.  The mixed
form keeps the masks and stays within its error bound of the same result: at
block size 64 it runs 4 digits (5 do not fit two pipeline stages in shared
memory), 1e-7 relative."""
import hashlib
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _inputs(g):
    """the fixture's inputs, rebuilt from its stored envelope table (exp may
    round differently in the last place on another host)"""
    from tests.golden.make_golden import CFG1, config1_inputs

    return CFG1, config1_inputs(g["env"])


def _sha(x):
    return hashlib.sha256(np.asfortranarray(x).tobytes(order="F")).hexdigest()


@pytest.fixture(scope="module")
def cfg1(api, ctx):
    g = np.load(os.path.join(GOLDEN, "config1_golden.npz"))
    c, (A, B) = _inputs(g)
    bs = c["bs"]
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    return c, g, gA, gB


def test_config1_matmult_fp64(api, ctx, cfg1):
    c, g, gA, gB = cfg1
    n, bs = c["n"], c["bs"]
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    nsig = api.matmult(gC, gA, 0, gB, 0, c["thresh"], 1.0, 0.0)
    assert nsig == int(g["mm_nsig"])
    assert np.array_equal(gC.mask(), g["mm_mask"])
    assert np.array_equal(gC.norms(), g["mm_norms"])
    assert _sha(gC.to_matrix()) == str(g["mm_sha256"])


def test_config1_dryrun_and_strassen_fp64(api, ctx, cfg1):
    c, g, gA, gB = cfg1
    n, bs = c["n"], c["bs"]
    levels, _ = api.matmult_strassen_dryrun(gA, gB, c["thresh"] * bs ** 3)
    tree = np.concatenate(levels).astype(np.uint8) if levels else np.zeros(0, np.uint8)
    assert np.array_equal(tree, g["tree"])
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    gC.fill_with_values(0.0)
    api.matmult_strassen_sparse(gC, gA, 0, gB, 0, c["thresh"], 1.0, 0.0, c["min_size"])
    out = gC.to_matrix()
    assert _sha(out) == str(g["st_sha256"])


def test_config1_mixed_form(api, ctx, cfg1):
    c, g, gA, gB = cfg1
    n, bs = c["n"], c["bs"]
    ref = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    api.matmult(ref, gA, 0, gB, 0, c["thresh"], 1.0, 0.0)
    R = ref.to_matrix()
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    nsig = api.matmult(gC, gA, 0, gB, 0, c["thresh"], 1.0, 0.0, form=api.FORM_OZAKI, n_digits=0)
    assert nsig == int(g["mm_nsig"])
    assert np.array_equal(gC.mask(), g["mm_mask"])
    assert np.linalg.norm(gC.to_matrix() - R) / np.linalg.norm(R) < 1e-7
    gS = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    gS.fill_with_values(0.0)
    api.matmult_strassen_sparse(gS, gA, 0, gB, 0, c["thresh"], 1.0, 0.0, c["min_size"], form=api.FORM_OZAKI,
                                n_digits=0)
    assert np.linalg.norm(gS.to_matrix() - R) / np.linalg.norm(R) < 1e-7


def test_config4_envelope_strassen_depths(api, ctx):
    """The large Strassen shape's envelope at n 2048 (dense core of the first
    512 rows and columns, exp(-|I-J|/10) tails, tau 1e-9): the dry-run tree,
    the screened matmult and matmult_strassen_sparse at depths 0..3 equal the
    compiled reference bit for bit."""
    from tests.golden.make_golden import CFG4S, config4s_inputs

    c = CFG4S
    g = np.load(os.path.join(GOLDEN, "config4s_golden.npz"))
    A, B = config4s_inputs(g["env"])
    n, bs, thr = c["n"], c["bs"], c["thresh"]
    gA = api.BlockSparseMatrix.from_dense(A, bs, bs, 0.0, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(B, bs, bs, 0.0, ctx=ctx)
    levels, _ = api.matmult_strassen_dryrun(gA, gB, thr * bs ** 3)
    tree = np.concatenate(levels).astype(np.uint8) if levels else np.zeros(0, np.uint8)
    assert np.array_equal(tree, g["tree"])
    gC = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
    assert api.matmult(gC, gA, 0, gB, 0, thr, 1.0, 0.0) == int(g["mm_nsig"])
    assert _sha(gC.to_matrix()) == str(g["mm_sha256"])
    for d in c["depths"]:
        gS = api.BlockSparseMatrix(n, n, bs, bs, 0.0, ctx=ctx)
        gS.fill_with_values(0.0)
        api.matmult_strassen_sparse(gS, gA, 0, gB, 0, thr, 1.0, 0.0, n >> d)
        assert _sha(gS.to_matrix()) == str(g[f"st_d{d}_sha256"]), f"depth {d}"
