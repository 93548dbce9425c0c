"""The CPU oracle, pinned against the reference's own outputs (CPU only).

Golden fixtures (tests/golden/, made by make_golden.py from the compiled
reference) hold the reference driver's printed norm, its K on the H2O
inputs, its 3c->2c result, and seeded matmult / Strassen / dry-run cases.
"""
import hashlib

import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits


def test_h2o_known_answer(oracle, h2o):
    """‖K‖_F printed by occ_ri_k_step.cpp:80 is 1.041507e+01."""
    d = h2o
    K = oracle.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 1)
    assert f"{np.linalg.norm(K):e}" == str(d["gold"]["driver_norm_line"])
    assert np.linalg.norm(K) == pytest.approx(10.415071322740426, rel=1e-14)
    assert same_bits(K, d["gold"]["K_part1"])


def test_h2o_partitions(oracle, h2o):
    d = h2o
    K4 = oracle.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 4)
    assert same_bits(K4, d["gold"]["K_part4"])
    Kd = oracle.rik_occ_dense(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 4)
    # the reference prints the sparse-vs-dense relative RMSD (occ_ri_k_step.cpp:129), ~1e-16
    assert np.linalg.norm(K4 - Kd) / np.linalg.norm(Kd) < 1e-14


def test_h2o_3c2c(oracle, h2o):
    d = h2o
    out = oracle.transform_3c2c(d["x3c"], d["v"], 3, 1e-20)
    assert same_bits(out, d["gold"]["X_PQm12"])
    # the reference's transformed integrals are this product (to 1e-14 relative)
    assert np.linalg.norm(out - d["ints"]) / np.linalg.norm(d["ints"]) < 1e-13


def _mm_inputs(cases, i):
    m, k, n, bs, tA, tB, al, be, cm, thr = cases[f"mm{i}_params"]
    m, k, n, bs, tA, tB, cm = int(m), int(k), int(n), int(bs), int(tA), int(tB), int(cm)
    ash = (k, m) if tA else (m, k)
    bsh = (n, k) if tB else (k, n)
    A = S.from_block_env(7, 3 * i, ash[0], ash[1], bs, cases[f"mm{i}_envA"])
    B = S.from_block_env(7, 3 * i + 1, bsh[0], bsh[1], bs, cases[f"mm{i}_envB"])
    Cin = S.gauss_matrix(7, 3 * i + 2, m, n)
    return dict(m=m, k=k, n=n, bs=bs, tA=tA, tB=tB, alpha=float(al), beta=float(be), c_mode=cm, thresh=float(thr),
                A=A, B=B, Cin=Cin)


@pytest.mark.parametrize("i", range(6))
def test_matmult_golden(oracle, ref_cases, i):
    p = _mm_inputs(ref_cases, i)
    bs = p["bs"]
    A = oracle.OBsm(*p["A"].shape, bs, bs, 1e-12, p["A"])
    B = oracle.OBsm(*p["B"].shape, bs, bs, 1e-12, p["B"])
    C = oracle.OBsm(p["m"], p["n"], bs, bs, 1e-3)
    if p["c_mode"] == 1:
        C.fill(0.0)
    if p["c_mode"] == 2:
        C.copy_from_dense(p["Cin"])
    oracle.matmult(C, A, p["tA"], B, p["tB"], p["thresh"], p["alpha"], p["beta"])
    assert same_bits(C.to_dense(), ref_cases[f"mm{i}_out"])
    assert np.array_equal(C.mask(), ref_cases[f"mm{i}_mask"])
    assert same_bits(C.norms(), ref_cases[f"mm{i}_norms"])


def _st_inputs(cases, i):
    n, bs, thr, ms = cases[f"st{i}_params"]
    n, bs, ms = int(n), int(bs), int(ms)
    env = cases[f"st{i}_env"]
    A = S.from_block_env(11, 2 * i, n, n, bs, env)
    B = S.from_block_env(11, 2 * i + 1, n, n, bs, env)
    return n, bs, float(thr), ms, A, B


@pytest.mark.parametrize("i", range(5))
def test_strassen_golden(oracle, ref_cases, i):
    n, bs, thr, ms, A, B = _st_inputs(ref_cases, i)
    Ao = oracle.OBsm(n, n, bs, bs, 0.0, A)
    Bo = oracle.OBsm(n, n, bs, bs, 0.0, B)
    levels, flops = oracle.strassen_dryrun(Ao, Bo, thr * bs ** 3)
    tree = np.concatenate(levels) if levels else np.zeros(0, np.uint8)
    assert np.array_equal(tree, ref_cases[f"st{i}_tree"])
    Co = oracle.OBsm(n, n, bs, bs, 0.0)
    Co.fill(0.0)
    oracle.matmult_strassen_sparse(Co, Ao, Bo, thr, ms)
    out = np.asfortranarray(Co.to_dense())
    assert hashlib.sha256(out.tobytes(order="F")).hexdigest() == str(ref_cases[f"st{i}_sha256"])


def test_strassen_engages(ref_cases):
    """the golden cases exercise Strassen nodes at more than one level"""
    assert any(ref_cases[f"st{i}_tree"].any() for i in range(5))


@pytest.mark.skipif("not __import__('oracle.oracle').oracle.ref_available()")
def test_oracle_vs_live_reference(oracle):
    """restatement == the compiled reference on fresh seeded inputs (where it
    was built)"""
    if oracle.ref() is None:
        pytest.skip("reference library not loadable here")
    for i, (m, k, n, bs, tA, tB) in enumerate([(50, 40, 30, 7, 0, 0), (40, 50, 30, 6, 1, 1), (64, 48, 80, 16, 1, 0)]):
        A = S.decay_matrix(3, 10 * i, k if tA else m, m if tA else k, bs, 1.5)
        B = S.decay_matrix(3, 10 * i + 1, n if tB else k, k if tB else n, bs, 1.5)
        out_r, mask_r, norms_r = oracle.ref_matmult(A, 1e-6, (bs, bs), B, 1e-6, (bs, bs), tA, tB, 1e-4, 1.0, 0.0)
        Ao = oracle.OBsm(*A.shape, bs, bs, 1e-6, A)
        Bo = oracle.OBsm(*B.shape, bs, bs, 1e-6, B)
        Co = oracle.OBsm(m, n, bs, bs, 0.0)
        oracle.matmult(Co, Ao, tA, Bo, tB, 1e-4, 1.0, 0.0)
        assert same_bits(Co.to_dense(), out_r)
        assert np.array_equal(Co.mask(), mask_r)
    for op in range(6):
        L_ = S.decay_matrix(5, op, 40, 40, 6, 2.0)
        R_ = S.decay_matrix(5, 10 + op, 40, 40, 6, 2.0)
        out_r, mask_r, norms_r, fro_r = oracle.ref_bsm_op(op, L_, 1e-3, R_, 1e-3, (6, 6), s=-0.75)
        Lo = oracle.OBsm(40, 40, 6, 6, 1e-3, L_)
        Ro = oracle.OBsm(40, 40, 6, 6, 1e-3, R_)
        [Lo.add, Lo.sub, Lo.add_transpose, lambda r: Lo.scale(-0.75), lambda r: Lo.recompress(),
         lambda r: Lo.calc_norms()][op](Ro)
        assert same_bits(Lo.to_dense(), out_r) and np.array_equal(Lo.mask(), mask_r)
        assert same_bits(Lo.norms(), norms_r) and Lo.frobenius_norm() == fro_r


def test_oracle_rejects_bad_keys(oracle, h2o):
    d = h2o
    keys = d["keys"].copy()
    keys[3] = d["n_bf"] ** 2
    with pytest.raises(ValueError):
        oracle.rik_occ_step(d["ints"], keys, d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 1)


# ---- symmetric K_mn on the occ step's mui_P ----

def _kmn_gold():
    import os

    from tests.conftest import GOLDEN
    return np.load(os.path.join(GOLDEN, "h2o_kmn_golden.npz"))


@pytest.mark.parametrize("n_part", [1, 4])
@pytest.mark.parametrize("tag,thr", [("t20", 1e-20), ("t6", 1e-6)])
def test_kmn_known_answer(oracle, h2o, n_part, tag, thr):
    """K_mn restatement == the same contraction on the compiled reference's
    classes (fixture), and exactly symmetric"""
    d = h2o
    K = oracle.rik_kmn_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, thr, n_part)
    assert same_bits(K, _kmn_gold()[f"Kmn_part{n_part}_{tag}"])
    assert np.array_equal(K, K.T)


def test_kmn_dense_formula(oracle, h2o):
    """at a negligible threshold K_mn = sum_P (U_P C)(U_P C)^T to rounding"""
    d = h2o
    n, keys = d["n_bf"], d["keys"].astype(np.int64)
    K = oracle.rik_kmn_step(d["ints"], d["keys"], d["c"], n, d["n_aux"], d["n_occ"], 3, 1e-20, 1)
    ref = np.zeros((n, n))
    for P in range(d["n_aux"]):
        U = np.zeros(n * n)
        U[keys] = d["ints"][:, P]
        m = U.reshape(n, n, order="F") @ d["c"]
        ref += m @ m.T
    assert np.linalg.norm(K - ref) / np.linalg.norm(ref) < 1e-13


def test_kmn_symmetric_u_identity(oracle):
    """for symmetric U_P the occ step's K_{mu j} = sum_P mui (ij + ji) equals
    2 K_mn C: ties the new contraction to the reference's own output"""
    rng = np.random.default_rng(3)
    n_bf, n_aux, n_occ, bs = 20, 9, 6, 4
    r, c = np.meshgrid(np.arange(n_bf), np.arange(n_bf), indexing="ij")
    keys = (r + c * n_bf).ravel(order="F").astype(np.uint64)
    ints = np.empty((n_bf * n_bf, n_aux), order="F")
    for P in range(n_aux):
        A = rng.standard_normal((n_bf, n_bf))
        ints[:, P] = (A + A.T).ravel(order="F")
    C = np.asfortranarray(rng.standard_normal((n_bf, n_occ)))
    K = oracle.rik_occ_step(ints, keys, C, n_bf, n_aux, n_occ, bs, 1e-30, 1)
    Kmn = oracle.rik_kmn_step(ints, keys, C, n_bf, n_aux, n_occ, bs, 1e-30, 1)
    assert np.linalg.norm(K - 2 * Kmn @ C) / np.linalg.norm(K) < 1e-13
