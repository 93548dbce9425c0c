"""Host logic of the screen comparison (strassen_gb300/screen.py): the
recount of the ij and K screens of occ_ri_k_step.cpp:107-116 against a
direct loop over block triples, and the flip report of two traces that
differ by one norm next to the threshold."""
import numpy as np

from strassen_gb300 import screen


def _trace(seed, n_aux=5, nb=4, nob=3, bs=4, thresh=1e-3):
    r = np.random.default_rng(seed)
    tr = {"mui_norm": 10.0 ** r.uniform(-4, 1, (n_aux, nb, nob)), "mui_flag": (r.random((n_aux, nb, nob)) < 0.8),
          "ij_flag": (r.random((n_aux, nob, nob)) < 0.7), "ijs_norm": 10.0 ** r.uniform(-4, 1, (n_aux, nob, nob)),
          "ijs_flag": (r.random((n_aux, nob, nob)) < 0.8), "c_norm": 10.0 ** r.uniform(-3, 1, (nb, nob)),
          "n_bf": nb * bs, "n_occ": nob * bs, "bs": bs, "thresh": thresh}
    for k in ("mui_flag", "ij_flag", "ijs_flag"):
        tr[k] = tr[k].astype(np.uint8)
    tr["ijs_norm"][0, 1, 2] = 0.0  # a block without its transpose partner keeps norm 0
    return tr


def _loop(tr):
    thr = tr["thresh"] * float(tr["bs"] ** 3)
    n, nb, nob = tr["mui_flag"].shape
    ij = k = 0
    for p in range(n):
        for a in range(nb):
            for i in range(nob):
                for j in range(nob):
                    if tr["mui_flag"][p, a, j] and tr["c_norm"][a, i] * tr["mui_norm"][p, a, j] >= thr:
                        ij += 1
                    if (tr["mui_flag"][p, a, i] and tr["ijs_flag"][p, i, j]
                            and tr["mui_norm"][p, a, i] * tr["ijs_norm"][p, i, j] >= thr):
                        k += 1
    return ij, k


def test_recount_matches_a_direct_loop():
    for seed in range(4):
        tr = _trace(seed)
        s = screen.survivors(tr, chunk=2)
        assert (s["ij"], s["K"]) == _loop(tr)


def test_identical_traces_have_no_flips():
    tr = _trace(7)
    c = screen.compare(tr, tr)
    for k in screen.PRODUCTS:
        assert c[k]["flips"] == 0 and c[k]["survivors_ref"] == c[k]["survivors_other"]
        assert c[k]["margin_min_all"] is not None and c[k]["margin_min_all"] >= 0
    assert all(v["differ"] == 0 for v in c["blocks"].values())


def test_one_norm_across_the_threshold_is_reported_with_its_margin():
    tr = _trace(3)
    thr = tr["thresh"] * tr["bs"] ** 3
    tr["mui_flag"][2, 1, 0] = 1
    tr["c_norm"][1, :] = 1.0
    tr["mui_norm"][2, 1, 0] = thr * (1 + 1e-12)  # survives, 1e-12 above the threshold
    other = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in tr.items()}
    other["mui_norm"][2, 1, 0] = thr * (1 - 1e-12)  # the same block in the other form: just below
    c = screen.compare(tr, other)
    nob = tr["mui_flag"].shape[2]
    # the ij triples (P 2, a 1, every ib, jb 0) flip; K triples through mui(2, 1, 0) may flip too
    assert c["ij"]["flips"] == nob
    assert 0 < c["ij"]["flip_margin_min"] < 2e-12
    assert c["ij"]["survivors_ref"] - c["ij"]["survivors_other"] == nob
    assert c["blocks"]["mui"]["differ"] == 0
    assert c["blocks"]["mui"]["norm_rel_diff_max"] > 1e-12
