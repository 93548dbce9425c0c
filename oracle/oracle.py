"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries, both built by ``oracle/build_ref.sh``:

* ``oracle/liboracle.so`` -- the plain-C restatement of the reference
  (``bsm_oracle.c``) on the deterministic BLAS shim (``naive_blas.c``);
* ``oracle/_ref/libref.so`` -- the reference's own headers compiled where they
  lie, behind ``ref_wrapper.cpp`` (only where the reference sources exist).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

c_size = C.c_size_t
c_dbl = C.c_double
c_int = C.c_int
c_vp = C.c_void_p
c_u8p = C.POINTER(C.c_uint8)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(c_vp)


def build():
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.ob_create.restype = c_vp
        L.ob_create.argtypes = [c_size, c_size, c_size, c_size, c_dbl]
        L.ob_free.argtypes = [c_vp]
        for n in ("ob_copy", "ob_add", "ob_sub", "ob_add_transpose"):
            getattr(L, n).argtypes = [c_vp, c_vp]
            getattr(L, n).restype = c_int
        L.ob_copy_from_dense.argtypes = [c_vp, c_vp]
        L.ob_copy_from_dense.restype = c_int
        L.ob_fill.argtypes = [c_vp, c_dbl]
        L.ob_zero.argtypes = [c_vp]
        L.ob_scale.argtypes = [c_vp, c_dbl]
        L.ob_calc_norms.argtypes = [c_vp]
        L.ob_recompress.argtypes = [c_vp]
        L.ob_frobenius_norm.argtypes = [c_vp]
        L.ob_frobenius_norm.restype = c_dbl
        L.ob_no_of_alloc_blocks.argtypes = [c_vp]
        L.ob_no_of_alloc_blocks.restype = c_size
        L.ob_to_dense.argtypes = [c_vp, c_vp]
        L.ob_get_mask.argtypes = [c_vp, c_vp]
        L.ob_get_norms.argtypes = [c_vp, c_vp]
        L.ob_dot.argtypes = [c_vp, c_vp, c_dbl]
        L.ob_dot.restype = c_dbl
        L.ob_matmult.argtypes = [c_vp, c_vp, c_int, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_vp]
        L.ob_matmult.restype = c_int
        L.ob_strassen_dryrun.argtypes = [c_vp, c_vp, c_dbl, C.POINTER(c_int), c_vp, c_size, c_vp]
        L.ob_strassen_dryrun.restype = c_int
        L.ob_matmult_strassen_sparse.argtypes = [c_vp, c_vp, c_vp, c_dbl, c_size]
        L.ob_matmult_strassen_sparse.restype = c_int
        L.ob_rik_occ_step.argtypes = [c_size, c_size, c_size, c_size, c_vp, c_vp, c_vp, c_size, c_dbl, c_int, c_vp]
        L.ob_rik_occ_step.restype = c_int
        L.ob_rik_kmn_step.argtypes = [c_size, c_size, c_size, c_size, c_vp, c_vp, c_vp, c_size, c_dbl, c_int, c_vp]
        L.ob_rik_kmn_step.restype = c_int
        L.ob_rik_occ_dense.argtypes = [c_size, c_size, c_size, c_size, c_vp, c_vp, c_vp, c_int, c_vp]
        L.ob_rik_occ_dense.restype = c_int
        L.ob_3c2c_transform.argtypes = [c_size, c_size, c_vp, c_vp, c_size, c_dbl, c_vp]
        L.ob_3c2c_transform.restype = c_int
        L.nb_enable_fast_gemm.argtypes = [C.c_char_p]
        L.nb_enable_fast_gemm.restype = c_int
        _LIB = L
    return _LIB


def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libref.so"))


def ref():
    """The compiled reference wrapper (None when it was not built here)."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            return None
        try:
            R = C.CDLL(path)
        except OSError:  # built for another architecture
            return None
        R.ref_matmult.argtypes = [c_size, c_size, c_vp, c_dbl, c_size, c_size, c_size, c_size, c_vp, c_dbl, c_size,
                                  c_size, c_int, c_int, c_int, c_dbl, c_vp, c_dbl, c_dbl, c_dbl, c_dbl, c_vp, c_vp,
                                  c_vp]
        R.ref_strassen.argtypes = [c_size, c_size, c_vp, c_vp, c_dbl, c_dbl, c_size, c_vp]
        R.ref_dryrun.argtypes = [c_size, c_size, c_vp, c_vp, c_dbl, c_dbl, C.POINTER(c_int), c_vp, c_size]
        R.ref_rik_occ_step.argtypes = [c_size, c_size, c_size, c_size, c_vp, c_vp, c_vp, c_size, c_dbl, c_int, c_vp]
        R.ref_rik_kmn_step.argtypes = [c_size, c_size, c_size, c_size, c_vp, c_vp, c_vp, c_size, c_dbl, c_int, c_vp]
        R.ref_bsm_op.argtypes = [c_int, c_size, c_size, c_size, c_size, c_vp, c_dbl, c_vp, c_dbl, c_dbl, c_vp, c_vp,
                                 c_vp, c_vp]
        _REF = R
    return _REF


def enable_fast_gemm(on=True):
    """Timing mode for the CPU baseline: dgemm through numpy's OpenBLAS."""
    L = lib()
    if not on:
        L.nb_enable_fast_gemm(None)
        return True
    libdir = os.path.join(os.path.dirname(np.__file__), "..", "numpy.libs")
    cands = [f for f in os.listdir(libdir) if f.startswith("libscipy_openblas")] if os.path.isdir(libdir) else []
    for f in cands:
        if L.nb_enable_fast_gemm(os.path.join(libdir, f).encode()) == 0:
            return True
    return False


class OBsm:
    """Oracle BlockSparseMatrix<double> (blocksparsematrix.h:19-93)."""

    def __init__(self, nr, nc, bsr, bsc, thresh, dense=None):
        self.L = lib()
        self.h = self.L.ob_create(nr, nc, bsr, bsc, thresh)
        self.nr, self.nc, self.bsr, self.bsc = nr, nc, bsr, bsc
        self.nrb = -(-nr // bsr) if nr else 0
        self.ncb = -(-nc // bsc) if nc else 0
        if dense is not None:
            self.copy_from_dense(dense)

    def __del__(self):
        try:
            self.L.ob_free(self.h)
        except Exception:
            pass

    def copy_from_dense(self, a):
        a = np.asfortranarray(a, dtype=np.float64)
        assert a.shape == (self.nr, self.nc)
        self.L.ob_copy_from_dense(self.h, _ptr(a))

    def to_dense(self):
        out = np.zeros((self.nr, self.nc), dtype=np.float64, order="F")
        self.L.ob_to_dense(self.h, _ptr(out))
        return out

    def mask(self):
        m = np.zeros(self.nrb * self.ncb, dtype=np.uint8)
        self.L.ob_get_mask(self.h, _ptr(m))
        return m

    def norms(self):
        n = np.zeros(self.nrb * self.ncb, dtype=np.float64)
        self.L.ob_get_norms(self.h, _ptr(n))
        return n

    def fill(self, v):
        self.L.ob_fill(self.h, v)

    def zero(self):
        self.L.ob_zero(self.h)

    def scale(self, s):
        self.L.ob_scale(self.h, s)

    def add(self, o):
        return self.L.ob_add(self.h, o.h)

    def sub(self, o):
        return self.L.ob_sub(self.h, o.h)

    def add_transpose(self, o):
        return self.L.ob_add_transpose(self.h, o.h)

    def copy_from(self, o):
        return self.L.ob_copy(self.h, o.h)

    def calc_norms(self):
        self.L.ob_calc_norms(self.h)

    def recompress(self):
        self.L.ob_recompress(self.h)

    def frobenius_norm(self):
        return self.L.ob_frobenius_norm(self.h)

    def no_of_alloc_blocks(self):
        return self.L.ob_no_of_alloc_blocks(self.h)


def matmult(C_, A, tA, B, tB, thresh, alpha=1.0, beta=0.0):
    nsig = np.zeros(1, dtype=np.uint64)
    st = lib().ob_matmult(C_.h, A.h, int(tA), B.h, int(tB), thresh, alpha, beta, _ptr(nsig))
    if st:
        raise ValueError(f"oracle matmult status {st}")
    return int(nsig[0])


def dot(A, B, thresh=0.0):
    return lib().ob_dot(A.h, B.h, thresh)


def strassen_dryrun(A, B, thresh_per_block):
    nb = A.nrb
    cap = sum(-(-nb // 2 ** (l + 1)) ** 3 for l in range(64) if 2 ** l <= 2 * nb) + 8
    tree = np.zeros(cap, dtype=np.uint8)
    flops = np.zeros(70, dtype=np.uint64)
    nl = c_int(0)
    st = lib().ob_strassen_dryrun(A.h, B.h, thresh_per_block, C.byref(nl), _ptr(tree), cap, _ptr(flops))
    if st:
        raise ValueError(f"oracle dryrun status {st}")
    levels, off = [], 0
    for l in range(nl.value):
        n = -(-nb // 2 ** (l + 1))
        levels.append(tree[off:off + n ** 3].copy())
        off += n ** 3
    return levels, flops[: nl.value + 1].copy()


def matmult_strassen_sparse(C_, A, B, thresh, min_size):
    st = lib().ob_matmult_strassen_sparse(C_.h, A.h, B.h, thresh, min_size)
    if st:
        raise ValueError(f"oracle strassen status {st}")


def rik_occ_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1):
    ints = np.asfortranarray(ints, dtype=np.float64)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    c_occ = np.asfortranarray(c_occ, dtype=np.float64)
    out = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
    st = lib().ob_rik_occ_step(n_bf, n_aux, n_occ, ints.shape[0], _ptr(ints), _ptr(keys), _ptr(c_occ), bs, thresh,
                               n_part, _ptr(out))
    if st:
        raise ValueError(f"oracle rik status {st}")
    return out


def rik_kmn_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1):
    """K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i) on the occ step's screened mui_P"""
    ints = np.asfortranarray(ints, dtype=np.float64)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    c_occ = np.asfortranarray(c_occ, dtype=np.float64)
    out = np.zeros((n_bf, n_bf), dtype=np.float64, order="F")
    st = lib().ob_rik_kmn_step(n_bf, n_aux, n_occ, ints.shape[0], _ptr(ints), _ptr(keys), _ptr(c_occ), bs, thresh,
                               n_part, _ptr(out))
    if st:
        raise ValueError(f"oracle rik kmn status {st}")
    return out


def rik_occ_dense(ints, keys, c_occ, n_bf, n_aux, n_occ, n_part=1):
    ints = np.asfortranarray(ints, dtype=np.float64)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    c_occ = np.asfortranarray(c_occ, dtype=np.float64)
    out = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
    st = lib().ob_rik_occ_dense(n_bf, n_aux, n_occ, ints.shape[0], _ptr(ints), _ptr(keys), _ptr(c_occ), n_part,
                                _ptr(out))
    if st:
        raise ValueError(f"oracle rik dense status {st}")
    return out


def transform_3c2c(ints_3c, v_m12, bs, thresh):
    X = np.asfortranarray(ints_3c, dtype=np.float64)
    V = np.asfortranarray(v_m12, dtype=np.float64)
    out = np.zeros(X.shape, dtype=np.float64, order="F")
    st = lib().ob_3c2c_transform(X.shape[0], X.shape[1], _ptr(X), _ptr(V), bs, thresh, _ptr(out))
    if st:
        raise ValueError(f"oracle 3c2c status {st}")
    return out


# ---- the compiled reference (only where it was built) ----

def ref_matmult(A, a_thresh, a_bs, B, b_thresh, b_bs, tA, tB, thresh, alpha, beta, c_mode=0, c_fill=0.0,
                c_in=None, c_thresh=0.0):
    R = ref()
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    cnr = A.shape[1] if tA else A.shape[0]
    cnc = B.shape[0] if tB else B.shape[1]
    cbr = a_bs[1] if tA else a_bs[0]
    cbc = b_bs[0] if tB else b_bs[1]
    nrb, ncb = -(-cnr // cbr), -(-cnc // cbc)
    out = np.zeros((cnr, cnc), dtype=np.float64, order="F")
    mask = np.zeros(nrb * ncb, dtype=np.uint8)
    norms = np.zeros(nrb * ncb, dtype=np.float64)
    cin = None if c_in is None else np.asfortranarray(c_in, dtype=np.float64)
    R.ref_matmult(A.shape[0], A.shape[1], _ptr(A), a_thresh, a_bs[0], a_bs[1], B.shape[0], B.shape[1], _ptr(B),
                  b_thresh, b_bs[0], b_bs[1], int(tA), int(tB), c_mode, c_fill, _ptr(cin), c_thresh, thresh, alpha,
                  beta, _ptr(out), _ptr(mask), _ptr(norms))
    return out, mask, norms


def ref_strassen(A, B, bs, in_thresh, thresh, min_size):
    R = ref()
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    out = np.zeros(A.shape, dtype=np.float64, order="F")
    R.ref_strassen(A.shape[0], bs, _ptr(A), _ptr(B), in_thresh, thresh, min_size, _ptr(out))
    return out


def ref_dryrun(A, B, bs, in_thresh, tpb):
    R = ref()
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    nb = -(-A.shape[0] // bs)
    cap = sum(-(-nb // 2 ** (l + 1)) ** 3 for l in range(64) if 2 ** l <= 2 * nb) + 8
    tree = np.zeros(cap, dtype=np.uint8)
    nl = c_int(0)
    R.ref_dryrun(A.shape[0], bs, _ptr(A), _ptr(B), in_thresh, tpb, C.byref(nl), _ptr(tree), cap)
    levels, off = [], 0
    for l in range(nl.value):
        n = -(-nb // 2 ** (l + 1))
        levels.append(tree[off:off + n ** 3].copy())
        off += n ** 3
    return levels


def ref_rik_occ_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1):
    R = ref()
    ints = np.asfortranarray(ints, dtype=np.float64)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    c_occ = np.asfortranarray(c_occ, dtype=np.float64)
    out = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
    R.ref_rik_occ_step(n_bf, n_aux, n_occ, ints.shape[0], _ptr(ints), _ptr(keys), _ptr(c_occ), bs, thresh, n_part,
                       _ptr(out))
    return out


def ref_rik_kmn_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1):
    R = ref()
    ints = np.asfortranarray(ints, dtype=np.float64)
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    c_occ = np.asfortranarray(c_occ, dtype=np.float64)
    out = np.zeros((n_bf, n_bf), dtype=np.float64, order="F")
    R.ref_rik_kmn_step(n_bf, n_aux, n_occ, ints.shape[0], _ptr(ints), _ptr(keys), _ptr(c_occ), bs, thresh, n_part,
                       _ptr(out))
    return out


def ref_bsm_op(op, lhs, lhs_thresh, rhs, rhs_thresh, bs, s=1.0):
    R = ref()
    lhs = np.asfortranarray(lhs, dtype=np.float64)
    rhs = np.asfortranarray(rhs, dtype=np.float64)
    nr, nc = lhs.shape
    nrb, ncb = -(-nr // bs[0]), -(-nc // bs[1])
    out = np.zeros((nr, nc), dtype=np.float64, order="F")
    mask = np.zeros(nrb * ncb, dtype=np.uint8)
    norms = np.zeros(nrb * ncb, dtype=np.float64)
    fro = np.zeros(1, dtype=np.float64)
    R.ref_bsm_op(op, nr, nc, bs[0], bs[1], _ptr(lhs), lhs_thresh, _ptr(rhs), rhs_thresh, s, _ptr(out), _ptr(mask),
                 _ptr(norms), _ptr(fro))
    return out, mask, norms, float(fro[0])
