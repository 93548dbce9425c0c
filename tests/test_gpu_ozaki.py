"""Ozaki split-precision form (bf16 digit slices on tcgen05, exact fp32 chains,
FP64 recombination) vs the FP64 form: identical screening (block masks,
surviving pairs), relative Frobenius error within the bound of the digit count.
"""
import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits

pytestmark = pytest.mark.gpu

# relative Frobenius error bounds per digit count (measured worst cases are
# about 30x below these on the seeded inputs)
BOUND = {2: 5e-3, 3: 5e-5, 4: 1e-7, 5: 1e-9, 6: 5e-12}


def _pair(api, ctx, m, k, n, bs, tA, tB, L, seed, thr_in=1e-9):
    ash = (k, m) if tA else (m, k)
    bsh = (n, k) if tB else (k, n)
    a = S.decay_matrix(seed, 1, ash[0], ash[1], bs, L)
    b = S.decay_matrix(seed, 2, bsh[0], bsh[1], bs, L)
    gA = api.BlockSparseMatrix.from_dense(a, bs, bs, thr_in, ctx=ctx)
    gB = api.BlockSparseMatrix.from_dense(b, bs, bs, thr_in, ctx=ctx)
    return gA, gB


@pytest.mark.parametrize("m,k,n,bs,tA,tB,alpha,beta,thr,L", [
    (240, 192, 216, 24, 0, 0, 1.0, 0.0, 1e-10, 0.8),
    (256, 256, 256, 64, 0, 0, 1.0, 0.0, 1e-10, 3.0),
    (128, 96, 160, 32, 1, 0, 1.0, 0.0, 1e-7, 0.5),
    (100, 77, 53, 9, 0, 1, -0.5, 1.0, 1e-6, 0.7),
    (160, 144, 96, 16, 0, 0, 2.0, 0.5, 1e-9, 1.5),
    (144, 192, 96, 48, 1, 1, 1.0, 0.0, 1e-9, 1.0),
    (1200, 1200, 240, 24, 0, 0, 1.0, 0.0, 1e-10, 4.0),
])
def test_ozaki_matches_fp64(api, ctx, m, k, n, bs, tA, tB, alpha, beta, thr, L):
    gA, gB = _pair(api, ctx, m, k, n, bs, tA, tB, L, 31)
    c0 = S.decay_matrix(31, 3, m, n, bs, L)
    C64 = api.BlockSparseMatrix.from_dense(c0, bs, bs, 1e-4, ctx=ctx)
    Coz = api.BlockSparseMatrix.from_dense(c0, bs, bs, 1e-4, ctx=ctx)
    n64 = api.matmult(C64, gA, tA, gB, tB, thr, alpha, beta)
    noz = api.matmult(Coz, gA, tA, gB, tB, thr, alpha, beta, form=api.FORM_OZAKI, n_digits=0)
    assert n64 == noz
    assert np.array_equal(C64.mask(), Coz.mask())
    r64, roz = C64.to_matrix(), Coz.to_matrix()
    err = np.linalg.norm(roz - r64) / np.linalg.norm(r64)
    nd = 5 if bs <= 48 else 4
    assert err < BOUND[nd], err


def test_ozaki_digit_ladder(api, ctx):
    """error falls by ~2^-8 per digit"""
    m = k = n = 480
    bs = 24
    gA, gB = _pair(api, ctx, m, k, n, bs, 0, 0, 2.0, 77)
    C64 = api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx)
    api.matmult(C64, gA, 0, gB, 0, 1e-12)
    ref = C64.to_matrix()
    errs = []
    for nd in (2, 3, 4, 5, 6):
        C = api.BlockSparseMatrix(m, n, bs, bs, 0.0, ctx=ctx)
        api.matmult(C, gA, 0, gB, 0, 1e-12, form=api.FORM_OZAKI, n_digits=nd)
        errs.append(np.linalg.norm(C.to_matrix() - ref) / np.linalg.norm(ref))
    print("digit ladder", errs)
    for nd, e in zip((2, 3, 4, 5, 6), errs):
        assert e < BOUND[nd], (nd, e)
    assert errs[0] > 50 * errs[1] > 50 * 50 * errs[2] > 50 * 50 * 50 * errs[3]


def test_ozaki_3c2c(api, ctx):
    s = S.RikSystem(seed=3, n_atoms=8, nbf=24, naux=30, n_occ=20, box=7.0)
    X, V = s.ints_3c(), s.v_m12()
    b64 = api.transform_3c2c(X, V, 24, 1e-10, ctx=ctx)
    # V^{-1/2} has condition 100, which amplifies the digit error: 6 digits
    errs = {}
    for nd in (5, 6):
        boz = api.transform_3c2c(X, V, 24, 1e-10, form=api.FORM_OZAKI, n_digits=nd, ctx=ctx)
        errs[nd] = np.linalg.norm(boz - b64) / np.linalg.norm(b64)
    print("3c2c digits", errs)
    assert errs[6] < 1e-10 and errs[5] < 1e-7


def test_ozaki_rejects_unsupported(api, ctx):
    gA, gB = _pair(api, ctx, 128, 128, 128, 64, 0, 0, 1.0, 5)
    C = api.BlockSparseMatrix(128, 128, 64, 64, 0.0, ctx=ctx)
    with pytest.raises(api.BsgError):
        api.matmult(C, gA, 0, gB, 0, 0.0, form=api.FORM_OZAKI, n_digits=9)
    with pytest.raises(api.BsgError):  # 6 digits of 64-wide blocks do not fit two pipeline stages
        api.matmult(C, gA, 0, gB, 0, 0.0, form=api.FORM_OZAKI, n_digits=6)


@pytest.mark.parametrize("nd", [5, 6])
def test_ozaki_rik_synthetic(api, ctx, nd):
    """occ-RI-K in the Ozaki form vs the FP64 form: same surviving block
    products (masks), K within 1e-9 relative"""
    s = S.RikSystem(seed=5, n_atoms=7, nbf=24, naux=20, n_occ=30, box=7.0)
    B = api.transform_3c2c(s.ints_3c(), s.v_m12(), 24, 1e-10, ctx=ctx)
    C = s.c_occ()
    K64, st64 = api.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, ctx=ctx, stats=True)
    Koz, stoz = api.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, form=api.FORM_OZAKI, n_digits=nd,
                                 p_chunk=32, ctx=ctx, stats=True)
    err = np.linalg.norm(Koz - K64) / np.linalg.norm(K64)
    print("rik ozaki digits", nd, err, st64[:3], stoz[:3])
    assert st64[:3] == stoz[:3]
    assert err < 1e-9


@pytest.mark.parametrize("n_occ,nbf,p_chunk", [(24, 24, 16), (60, 24, 16), (77, 24, 16), (50, 22, 7)])
def test_ozaki_rik_column_pairs(api, ctx, n_occ, nbf, p_chunk):
    """occupied block columns paired on the N side of the ij and K products
    and aux functions paired on the N side of mui: an odd number of column
    blocks (the last pair half empty), ragged last blocks, a single block,
    ragged basis blocks and odd chunks of aux functions (the last pair a
    single one); masks and K as in the FP64 form"""
    s = S.RikSystem(seed=12, n_atoms=6, nbf=nbf, naux=10, n_occ=n_occ, box=6.5)
    B = api.transform_3c2c(s.ints_3c(), s.v_m12(), 24, 1e-10, ctx=ctx)
    C = s.c_occ()
    K64, st64 = api.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, ctx=ctx, stats=True)
    Koz, stoz = api.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, form=api.FORM_OZAKI,
                                 n_digits=5, p_chunk=p_chunk, ctx=ctx, stats=True)
    err = np.linalg.norm(Koz - K64) / np.linalg.norm(K64)
    print("column pairs", n_occ, err, st64[:3], stoz[:3])
    assert st64[:3] == stoz[:3]
    assert err < 1e-9


def test_ozaki_rik_h2o(api, ctx, h2o):
    d = h2o
    K = api.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20,
                         form=api.FORM_OZAKI, n_digits=5, ctx=ctx)
    ref = d["gold"]["K_part1"]
    assert np.linalg.norm(K - ref) / np.linalg.norm(ref) < 1e-9


def test_ozaki_pipeline(api, ctx):
    """3c->2c (6 digits) then occ-RI-K (5 digits) against the FP64 pipeline"""
    s = S.RikSystem(seed=8, n_atoms=8, nbf=24, naux=24, n_occ=40, box=8.0)
    X, V, C = s.ints_3c(), s.v_m12(), s.c_occ()
    B64 = api.transform_3c2c(X, V, 24, 1e-10, ctx=ctx)
    K64 = api.rik_occ_step(B64, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, ctx=ctx)
    Boz = api.transform_3c2c(X, V, 24, 1e-10, form=api.FORM_OZAKI, n_digits=6, ctx=ctx)
    Koz = api.rik_occ_step(Boz, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, form=api.FORM_OZAKI, n_digits=5,
                           ctx=ctx)
    err = np.linalg.norm(Koz - K64) / np.linalg.norm(K64)
    print("pipeline error", err)
    assert err < 1e-9


@pytest.mark.parametrize("pinned", [False, True, "interior"])
@pytest.mark.parametrize("nd,tol", [(6, 1e-10), (5, 1e-7)])
@pytest.mark.parametrize("n_atoms,bs", [(8, 24), (3, 16), (1, 24)])
def test_3c2c_host_upload_matches_device(api, ctx, n_atoms, bs, nd, tol, pinned):
    """host integrals stream in by row ranges overlapping the transform: the
    output equals the device-input transform bit for bit (ranges of whole
    block rows, a ragged last range, and a single range); at 5 digits the
    tiles carry two X block rows (split into exact rectangles).  Pageable
    host memory goes through the copy engine, pinned memory is read by SMs
    beside the GEMM launches (one atom: 299 rows, odd, so 8-byte loads)"""
    torch = pytest.importorskip("torch")
    s = S.RikSystem(seed=4, n_atoms=n_atoms, nbf=24, naux=12, n_occ=10, box=5.0)
    X, V = s.ints_3c(), s.v_m12()
    if n_atoms == 1:
        X = np.asfortranarray(X[:-1])
    if pinned == "interior":
        # the matrix starts one column into a larger pinned allocation
        Xp = torch.zeros((X.shape[1] + 1, X.shape[0]), dtype=torch.float64).pin_memory()
        Xp[1:] = torch.from_numpy(np.ascontiguousarray(X.T))
        X = Xp[1:].numpy().T
    elif pinned:
        Xp = torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory()
        X = Xp.numpy().T  # the same column-major matrix in pinned memory
    out_h = api.transform_3c2c(X, V, bs, 1e-10, form=api.FORM_OZAKI, n_digits=nd, ctx=ctx)
    Xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda().T
    Vd = torch.from_numpy(np.ascontiguousarray(V.T)).cuda().T
    out_d = torch.zeros((X.shape[1], X.shape[0]), dtype=torch.float64, device="cuda").T
    api.transform_3c2c(Xd, Vd, bs, 1e-10, form=api.FORM_OZAKI, n_digits=nd, out=out_d, ctx=ctx)
    assert same_bits(out_h, out_d.cpu().numpy())
    ref = api.transform_3c2c(X, V, bs, 1e-10, ctx=ctx)
    assert np.linalg.norm(out_h - ref) / np.linalg.norm(ref) < tol
