"""Symmetric exchange matrix K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i) on the GPU.

FP64 form: bit-identical to the contraction built on the compiled
reference's classes (H2O fixture) and to the oracle on synthetic systems,
with the occ step's K from the same pass unchanged.  Mixed form: within
1e-9 of the FP64 form with the same surviving block products."""
import os

import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import GOLDEN, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kmn_gold():
    return np.load(os.path.join(GOLDEN, "h2o_kmn_golden.npz"))


@pytest.mark.parametrize("n_part", [1, 4])
@pytest.mark.parametrize("tag,thr", [("t20", 1e-20), ("t6", 1e-6)])
def test_h2o_known_answer(api, ctx, h2o, kmn_gold, n_part, tag, thr):
    d = h2o
    Kmn = api.rik_kmn_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, thr, n_part=n_part,
                           ctx=ctx)
    assert same_bits(Kmn, kmn_gold[f"Kmn_part{n_part}_{tag}"])
    assert np.array_equal(Kmn, Kmn.T)


@pytest.mark.parametrize("p_chunk", [1, 7, 50])
def test_h2o_both_outputs(api, ctx, h2o, kmn_gold, p_chunk):
    """one pass gives K_mn and the occ step's K, both bit-identical, across
    chunk boundaries that cut through partitions"""
    d = h2o
    Kmn, K, st = api.rik_kmn_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20,
                                  n_part=4, p_chunk=p_chunk, k_out=True, ctx=ctx, stats=True)
    assert same_bits(Kmn, kmn_gold["Kmn_part4_t20"])
    assert same_bits(K, d["gold"]["K_part4"])
    _, st0 = api.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part=4,
                              ctx=ctx, stats=True)
    assert st[:5] == st0 and st[5] > 0


@pytest.mark.parametrize("params", [dict(n_atoms=6, nbf=8, naux=10, n_occ=10, box=5.0, bs=8, thresh=1e-10, n_part=1),
                                    dict(n_atoms=7, nbf=6, naux=9, n_occ=13, box=6.0, bs=6, thresh=1e-8, n_part=3),
                                    dict(n_atoms=5, nbf=24, naux=12, n_occ=20, box=8.0, bs=24, thresh=1e-10, n_part=2)])
def test_synthetic_vs_oracle(api, oracle, ctx, params):
    p = dict(params)
    bs, thr, npart = p.pop("bs"), p.pop("thresh"), p.pop("n_part")
    s = S.RikSystem(seed=6, **p)
    B = oracle.transform_3c2c(s.ints_3c(), s.v_m12(), bs, thr)
    C = s.c_occ()
    Ko = oracle.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, thr, npart)
    Kg = api.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, thr, n_part=npart, p_chunk=4, ctx=ctx)
    assert same_bits(Kg, Ko)


def test_device_inputs_and_outputs(api, ctx, h2o, kmn_gold):
    torch = pytest.importorskip("torch")
    d = h2o
    ints = torch.from_numpy(np.ascontiguousarray(d["ints"].T)).cuda().T
    keys = torch.from_numpy(d["keys"].view(np.int64)).cuda()
    c = torch.from_numpy(np.ascontiguousarray(d["c"].T)).cuda().T
    out = torch.zeros((d["n_bf"], d["n_bf"]), dtype=torch.float64, device="cuda")
    Kmn, K = api.rik_kmn_step(ints, keys, c, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, out=out, k_out=True,
                              ctx=ctx)
    assert same_bits(Kmn.cpu().numpy().T, kmn_gold["Kmn_part1_t20"])
    assert same_bits(K.cpu().numpy(), d["gold"]["K_part1"])


def test_empty_aux_and_null_output(api, ctx, h2o):
    d = h2o
    Kmn = api.rik_kmn_step(d["ints"][:, :0], d["keys"], d["c"], d["n_bf"], 0, d["n_occ"], 3, 1e-20, ctx=ctx)
    assert Kmn.shape == (d["n_bf"], d["n_bf"]) and not Kmn.any()
    assert api.lib.bsg_rik_kmn_step(ctx.h, None, None, None, 0, None) != 0


@pytest.mark.parametrize("bs,nd,tol", [(24, 5, 1e-9), (32, 5, 1e-9), (64, 4, 1e-7)])
def test_mixed_form(api, ctx, bs, nd, tol):
    """mixed form: same surviving block products as the FP64 form, K_mn
    within tol relative (1e-9 at 5 digits; 64-wide blocks fit 4 digits in
    shared memory), exactly symmetric, and the K from the same pass within tol
    too; ragged blocks (n_occ and n_bf not multiples of bs)"""
    s = S.RikSystem(seed=9, n_atoms=7, nbf=20, naux=14, n_occ=45, box=7.0)
    B = api.transform_3c2c(s.ints_3c(), s.v_m12(), bs, 1e-10, ctx=ctx)
    C = s.c_occ()
    K64m, K64, st64 = api.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, 1e-10, k_out=True, ctx=ctx,
                                       stats=True)
    Kozm, Koz, stoz = api.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, 1e-10, form=api.FORM_OZAKI,
                                       n_digits=nd, p_chunk=20, k_out=True, ctx=ctx, stats=True)
    em = np.linalg.norm(Kozm - K64m) / np.linalg.norm(K64m)
    ek = np.linalg.norm(Koz - K64) / np.linalg.norm(K64)
    print("kmn mixed", bs, nd, em, ek, st64, stoz)
    assert np.array_equal(Kozm, Kozm.T)
    assert st64[0] == stoz[0] and st64[5] == stoz[5]
    assert em < tol and ek < tol


@pytest.mark.parametrize("n_atoms,p_chunk", [(6, 0), (5, 7)])
def test_mixed_kmn_only(api, ctx, n_atoms, p_chunk):
    """K_mn without the occ step's K (the ij and K products are skipped);
    an odd number of basis block rows leaves the last N-side pair half empty"""
    s = S.RikSystem(seed=10, n_atoms=n_atoms, nbf=24, naux=12, n_occ=30, box=6.0)
    B = api.transform_3c2c(s.ints_3c(), s.v_m12(), 24, 1e-10, ctx=ctx)
    C = s.c_occ()
    K64 = api.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, ctx=ctx)
    Koz, st = api.rik_kmn_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, form=api.FORM_OZAKI, n_digits=5,
                               p_chunk=p_chunk, ctx=ctx, stats=True)
    assert np.array_equal(Koz, Koz.T)
    assert st[1] == 0 and st[2] == 0 and st[5] > 0
    assert np.linalg.norm(Koz - K64) / np.linalg.norm(K64) < 1e-9
