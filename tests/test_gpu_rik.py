"""occ-RI-K step and 3c->2c transform on the GPU, FP64 form: bit-identical to
the reference (golden H2O outputs) and to the oracle on synthetic systems."""
import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_part", [1, 4])
def test_h2o_known_answer(api, ctx, h2o, n_part):
    d = h2o
    K = api.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part=n_part,
                         ctx=ctx)
    assert same_bits(K, d["gold"][f"K_part{n_part}"])
    assert f"{np.linalg.norm(K):e}" == str(d["gold"]["driver_norm_line"])


@pytest.mark.parametrize("p_chunk", [1, 7, 50])
def test_h2o_chunking(api, ctx, h2o, p_chunk):
    """chunk boundaries that cut through partitions do not change the order"""
    d = h2o
    K = api.rik_occ_step(d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part=4,
                         p_chunk=p_chunk, ctx=ctx)
    assert same_bits(K, d["gold"]["K_part4"])


def test_h2o_3c2c(api, ctx, h2o):
    d = h2o
    out = api.transform_3c2c(d["x3c"], d["v"], 3, 1e-20, ctx=ctx)
    assert same_bits(out, d["gold"]["X_PQm12"])


@pytest.mark.parametrize("params", [dict(n_atoms=6, nbf=8, naux=10, n_occ=10, box=5.0, bs=8, thresh=1e-10, n_part=1),
                                    dict(n_atoms=7, nbf=6, naux=9, n_occ=13, box=6.0, bs=6, thresh=1e-8, n_part=3),
                                    dict(n_atoms=5, nbf=24, naux=12, n_occ=20, box=8.0, bs=24, thresh=1e-10, n_part=2)])
def test_synthetic_vs_oracle(api, oracle, ctx, params):
    p = dict(params)
    bs, thr, npart = p.pop("bs"), p.pop("thresh"), p.pop("n_part")
    s = S.RikSystem(seed=5, **p)
    X = s.ints_3c()
    V = s.v_m12()
    C = s.c_occ()
    B = oracle.transform_3c2c(X, V, bs, thr)
    Bg = api.transform_3c2c(X, V, bs, thr, ctx=ctx)
    assert same_bits(Bg, B)
    Ko = oracle.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, thr, npart)
    Kg, st = api.rik_occ_step(B, s.keys, C, s.n_bf, s.n_aux, s.n_occ, bs, thr, n_part=npart, ctx=ctx, stats=True)
    assert same_bits(Kg, Ko)
    assert st[0] > 0 and st[1] > 0 and st[2] > 0


def test_device_inputs(api, ctx, h2o):
    torch = pytest.importorskip("torch")
    d = h2o
    ints = torch.from_numpy(np.ascontiguousarray(d["ints"].T)).cuda().T
    keys = torch.from_numpy(d["keys"].view(np.int64)).cuda()
    c = torch.from_numpy(np.ascontiguousarray(d["c"].T)).cuda().T
    out = torch.zeros((d["n_occ"], d["n_bf"]), dtype=torch.float64, device="cuda").T
    api.rik_occ_step(ints, keys, c, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part=1, out=out, ctx=ctx)
    assert same_bits(out.cpu().numpy(), d["gold"]["K_part1"])


def test_bad_key_rejected(api, ctx, h2o):
    d = h2o
    keys = d["keys"].copy()
    keys[5] = d["n_bf"] ** 2
    with pytest.raises(api.BsgError) as e:
        api.rik_occ_step(d["ints"], keys, d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, ctx=ctx)
    assert e.value.code == 1


def test_empty_aux(api, ctx, h2o):
    d = h2o
    K = api.rik_occ_step(d["ints"][:, :0], d["keys"], d["c"], d["n_bf"], 0, d["n_occ"], 3, 1e-20, ctx=ctx)
    assert not K.any()
