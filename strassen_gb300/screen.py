"""Screening masks of the occ-RI-K step, recounted on the host from a screen
trace (``api.rik_occ_step(..., trace=True)``), and the comparison of the
traces of two arithmetic forms.

The screened products of occ_ri_k_step.cpp:107-116 keep a block triple when
``||A_ik|| * ||B_kj|| >= thresh * bs^3`` (blocksparsematrix.hpp:391-397):

* ``mui_P = U_P C``: norms of the inputs only, so its block structure is the
  same in every form;
* ``ij_P = C^T mui_P``: C norms times the norms of the computed mui_P blocks
  (mui_P.calc_frobenius_norms(), :108);
* ``K += mui_P ijs_P``: mui_P norms times the ijs_P norms refreshed by
  add_transpose (:113, blocksparsematrix.hpp:244).

The norms of computed blocks differ between the FP64 and the mixed form in
their last digits, so a triple whose norm product lies within that difference
of the threshold can survive in one form and not in the other: a flip.  Each
flip is reported with its margin ``|est - thr| / thr`` (est from the first
trace, the FP64 form), next to the smallest margin of all triples (how close
the closest call was).
"""
from __future__ import annotations

import numpy as np

PRODUCTS = ("ij", "K")


def _triples(tr, p0, p1):
    """norm products and keep decisions of the ij and K triples of aux
    functions p0..p1: ij [P, a, ib, jb], K [P, a, ib, jb]"""
    thr = tr["thresh"] * float(tr["bs"] ** 3)
    mn = np.where(tr["mui_flag"][p0:p1] != 0, tr["mui_norm"][p0:p1], 0.0)  # [P, a, j]
    mf = tr["mui_flag"][p0:p1] != 0
    cn = tr["c_norm"]  # [a, i]
    # ij_P(ib, jb) over a: ||C(a, ib)|| * ||mui_P(a, jb)||
    est_ij = cn[None, :, :, None] * mn[:, :, None, :]
    live_ij = mf[:, :, None, :] & np.ones_like(cn, dtype=bool)[None, :, :, None]
    keep_ij = live_ij & (est_ij >= thr)
    # K(a, jb) over (P, ib): ||mui_P(a, ib)|| * ||ijs_P(ib, jb)||
    sf = tr["ijs_flag"][p0:p1] != 0
    sn = np.where(sf, tr["ijs_norm"][p0:p1], 0.0)  # [P, i, j]
    est_k = mn[:, :, :, None] * sn[:, None, :, :]
    live_k = mf[:, :, :, None] & sf[:, None, :, :]
    keep_k = live_k & (est_k >= thr)
    return thr, {"ij": (est_ij, live_ij, keep_ij), "K": (est_k, live_k, keep_k)}


def survivors(tr, chunk=256):
    """surviving triples of the ij and K products recounted from one trace
    (equal to the step's own counters stats[1], stats[2])"""
    n = tr["mui_flag"].shape[0]
    out = {k: 0 for k in PRODUCTS}
    for p0 in range(0, n, chunk):
        _, t = _triples(tr, p0, min(n, p0 + chunk))
        for k in PRODUCTS:
            out[k] += int(t[k][2].sum())
    return out


def compare(tr_ref, tr_other, chunk=256):
    """Per product: surviving triples in both traces, the flips between them
    with the smallest and largest margin among the flips, the smallest margin
    of every live triple of the reference trace, and the block-level mask
    differences of mui_P, ij_P and ijs_P (presence) with the largest relative
    difference of the norms both forms computed."""
    n = tr_ref["mui_flag"].shape[0]
    assert tr_other["mui_flag"].shape == tr_ref["mui_flag"].shape
    res = {k: {"survivors_ref": 0, "survivors_other": 0, "flips": 0, "flip_margin_min": None,
               "flip_margin_max": None, "margin_min_all": None} for k in PRODUCTS}
    for p0 in range(0, n, chunk):
        p1 = min(n, p0 + chunk)
        thr, a = _triples(tr_ref, p0, p1)
        _, b = _triples(tr_other, p0, p1)
        for k in PRODUCTS:
            est, live, keep = a[k]
            keep_o = b[k][2]
            r = res[k]
            r["survivors_ref"] += int(keep.sum())
            r["survivors_other"] += int(keep_o.sum())
            flip = keep != keep_o
            margin = np.abs(est - thr) / thr
            if flip.any():
                fm = margin[flip]
                r["flips"] += int(flip.sum())
                r["flip_margin_min"] = float(min(fm.min(), r["flip_margin_min"] or np.inf))
                r["flip_margin_max"] = float(max(fm.max(), r["flip_margin_max"] or 0.0))
            if live.any():
                m = float(margin[live].min())
                r["margin_min_all"] = m if r["margin_min_all"] is None else min(m, r["margin_min_all"])
    blocks = {}
    for name in ("mui", "ij", "ijs"):
        fa, fb = tr_ref[name + "_flag"] != 0, tr_other[name + "_flag"] != 0
        d = {"present_ref": int(fa.sum()), "present_other": int(fb.sum()), "differ": int((fa != fb).sum())}
        if name + "_norm" in tr_ref:
            both = fa & fb & (tr_ref[name + "_norm"] != 0)
            if both.any():
                x, y = tr_ref[name + "_norm"][both], tr_other[name + "_norm"][both]
                d["norm_rel_diff_max"] = float(np.max(np.abs(x - y) / np.abs(x)))
        blocks[name] = d
    res["blocks"] = blocks
    return res
