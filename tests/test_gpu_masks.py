"""Per-block screening masks of the mixed form against the FP64 form.

The occ-RI-K step screens on norms of computed intermediates: mui_P's norms
(occ_ri_k_step.cpp:108) decide which ij_P triples survive, and ijs_P's norms
(add_transpose, blocksparsematrix.hpp:244) which K triples survive.  Both
forms run with the screen trace on the same transformed integrals; the trace
is recounted on the host (strassen_gb300/screen.py), which must reproduce the
step's own surviving-product counters exactly, and the forms are compared
block by block and triple by triple: mui_P's structure depends on the inputs
only and must be identical; a triple of ij or K may flip only where its norm
product lies within the mixed form's norm error of the threshold.
"""
import numpy as np
import pytest

from strassen_gb300 import screen
from strassen_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _system(n_atoms):
    box = 12.0 * (n_atoms / 40) ** (1.0 / 3.0)  # the 40-atom workload's density
    return S.RikSystem(seed=42, n_atoms=n_atoms, nbf=24, naux=84, n_occ=5 * n_atoms, box=box)


@pytest.mark.parametrize("thresh", [1e-10, 1e-6])
def test_masks_mixed_vs_fp64_same_integrals(api, ctx, thresh):
    import torch

    s = _system(12)
    dev = torch.device("cuda", 0)
    X = s.ints_3c_torch(dev).T
    V = torch.from_numpy(np.ascontiguousarray(s.v_m12().T)).to(dev).T
    C = torch.from_numpy(np.ascontiguousarray(s.c_occ().T)).to(dev).T
    keys = torch.from_numpy(s.keys.view(np.int64)).to(dev)
    B = torch.empty((s.n_aux, s.n_vec2), dtype=torch.float64, device=dev).T
    api.transform_3c2c(X, V, 24, thresh, out=B, ctx=ctx)
    res = {}
    for form in (api.FORM_FP64, api.FORM_OZAKI):
        K, st, tr = api.rik_occ_step(B, keys, C, s.n_bf, s.n_aux, s.n_occ, 24, thresh, form=form, n_digits=5,
                                     ctx=ctx, trace=True)
        rc = screen.survivors(tr)
        # the host recount is the device screen, triple for triple
        assert (rc["ij"], rc["K"]) == (st[1], st[2])
        res[form] = (np.asarray(K.cpu() if hasattr(K, "cpu") else K), st, tr)
    (K64, st64, tr64), (Koz, stoz, troz) = res[api.FORM_FP64], res[api.FORM_OZAKI]
    c = screen.compare(tr64, troz)
    assert st64[0] == stoz[0], "mui = U C screens on input norms only"
    assert c["blocks"]["mui"]["differ"] == 0
    assert c["blocks"]["mui"]["norm_rel_diff_max"] < 1e-9
    for k in screen.PRODUCTS:
        if c[k]["flips"]:
            assert c[k]["flip_margin_max"] < 1e-8, (k, c[k])
    # without flips the masks of ij and ijs are identical block by block
    if c["ij"]["flips"] == 0:
        assert c["blocks"]["ij"]["differ"] == 0 and c["blocks"]["ijs"]["differ"] == 0
        assert st64[1] == stoz[1] and st64[3:] == stoz[3:]
    assert np.linalg.norm(Koz - K64) / np.linalg.norm(K64) < 1e-9
