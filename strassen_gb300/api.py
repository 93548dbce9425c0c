"""Python mirror of the reference's interface over libbsgpu.so.

Names and argument meaning follow the reference's C++ API:

* :class:`BlockMemoryPool`   -- blockallocator.h:8-25
* :class:`BlockSparseMatrix` -- blocksparsematrix.h:19-93
* :func:`matmult`            -- blocksparsematrix.h:96-99
* :func:`dot`                -- blocksparsematrix.h:102
* :func:`matmult_strassen_sparse`, :func:`matmult_strassen_dryrun` -- strassen.hpp:511,688
* :func:`tensormult_contract`, :func:`tensormult_batched` -- blocksparse3d_tensor.h:11-24
* :func:`rik_occ_step`       -- occ_ri_k_step.cpp:83-130
* :func:`rik_kmn_step`       -- symmetric K_mn on the same step's mui_P (:102-108)
* :func:`transform_3c2c`     -- 3c_2c_transform.cpp:44-57

Errors the reference turns into assert/exit(1) raise :class:`BsgError`.
Dense arrays are column-major float64; numpy arrays live on the host, torch
CUDA tensors on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import BSG_DEVICE, BSG_HOST, FORM_FP64, FORM_OZAKI, BsgError, RikArgs, ScreenTrace, check, lib  # noqa: F401
from ._lib import (SCHED_COST, SCHED_DENSE, SCHED_FEATURES, SCHED_MLP, SCHED_NODE_FEATURES, SCHED_NONE,  # noqa: F401
                   SCHED_OPTIONS, SCHED_ROOT)

_DEFAULT_CTX = None


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _buf(a, dtype=np.float64):
    """(pointer, where, keepalive) for a host numpy array or a CUDA tensor.

    A context's stream does not wait for torch's streams, so the work torch
    has queued on the current stream (the kernels that produce the tensor)
    is finished first: otherwise the library could read a tensor that is
    still being written.  Where the context runs on torch's current stream
    the stream is already in order and the wait returns at once."""
    if a is None:
        return None, BSG_HOST, None
    if _is_device(a):
        import torch

        torch.cuda.current_stream(a.device).synchronize()
        return C.c_void_p(a.data_ptr()), BSG_DEVICE, a
    if hasattr(a, "data_ptr"):  # CPU torch tensor
        a = a.numpy()
    arr = np.asfortranarray(a, dtype=dtype)
    return arr.ctypes.data_as(C.c_void_p), BSG_HOST, arr


class Context:
    """A device plus the CUDA stream every call on it is ordered on."""

    def __init__(self, device=0, stream=None):
        h = C.c_void_p()
        check(lib.bsg_ctx_create(device, stream, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            lib.bsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(lib.bsg_ctx_sync(self.h))

    def launch_count(self):
        n = C.c_uint64()
        check(lib.bsg_ctx_launch_count(self.h, C.byref(n)))
        return n.value

    def set_timing(self, on=True):
        """CUDA-event timing of the tensor-core GEMM launches (resets totals)"""
        check(lib.bsg_ctx_set_timing(self.h, int(bool(on))))

    def gemm_timing(self):
        """(launches, milliseconds, unpadded FP64-equivalent multiply-adds)"""
        n, ms, macs = C.c_uint64(), C.c_double(), C.c_double()
        check(lib.bsg_ctx_gemm_timing(self.h, C.byref(n), C.byref(ms), C.byref(macs)))
        return n.value, ms.value, macs.value

    def set_autotune(self, on=True, forget=False):
        """switch the tensor-core GEMM's autotuner on or off (forget: drop its cache)"""
        check(lib.bsg_ctx_set_autotune(self.h, -1 if forget else int(bool(on))))

    def autotune_entries(self):
        """cached tuning decisions: (mp, kp, np, digits) -> (slots per tile, stages)"""
        n = C.c_int()
        check(lib.bsg_ctx_autotune_entries(self.h, None, 0, C.byref(n)))
        buf = np.zeros(6 * max(n.value, 1), np.int32)
        check(lib.bsg_ctx_autotune_entries(self.h, buf.ctypes.data, n.value, C.byref(n)))
        e = buf[:6 * n.value].reshape(-1, 6)
        return {tuple(int(x) for x in r[:4]): (int(r[4]), int(r[5])) for r in e}

    STALL_KEYS = ("mma_wait_operands", "mma_wait_accumulator", "mma_total", "producer_wait_stage",
                  "epilogue_wait_chain", "epilogue_drain", "epilogue_store", "steps", "mmas", "copied_steps",
                  "live_pairs", "pair_capacity")

    def gemm_stalls(self):
        """stall breakdown of the timed tensor-core GEMM launches (SM cycles summed over CTAs)"""
        out = (C.c_uint64 * 12)()
        check(lib.bsg_ctx_gemm_stalls(self.h, out))
        return dict(zip(self.STALL_KEYS, list(out)))


def default_context():
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context(0)
    return _DEFAULT_CTX


class BlockMemoryPool:
    """Device block pool shared by the matrices created on it."""

    def __init__(self, block_elems, ctx=None, _handle=None):
        self.ctx = ctx or default_context()
        if _handle is not None:
            self.h = _handle
        else:
            h = C.c_void_p()
            check(lib.bsg_pool_create(self.ctx.h, block_elems, C.byref(h)))
            self.h = h

    def __del__(self):
        try:
            lib.bsg_pool_release(self.h)
        except Exception:
            pass

    def adjust_blocksize(self, n):
        check(lib.bsg_pool_adjust_blocksize(self.h, n))

    def release_all_memory(self):
        check(lib.bsg_pool_release_all_memory(self.h))

    def stats(self):
        t, f, b = C.c_size_t(), C.c_size_t(), C.c_size_t()
        check(lib.bsg_pool_stats(self.h, C.byref(t), C.byref(f), C.byref(b)))
        return {"blocks_total": t.value, "blocks_free": f.value, "bytes": b.value}


class BlockSparseMatrix:
    """BlockSparseMatrix<double>: a grid of dense blocks in a device pool."""

    def __init__(self, nr, nc, bsr, bsc, thresh, pool=None, ctx=None, dense=None):
        self.ctx = ctx or (pool.ctx if pool is not None else default_context())
        h = C.c_void_p()
        check(lib.bsg_bsm_create(self.ctx.h, nr, nc, bsr, bsc, float(thresh), pool.h if pool else None, C.byref(h)))
        self.h = h
        self.nr, self.nc, self.bsr, self.bsc = nr, nc, bsr, bsc
        self.nrb = -(-nr // bsr) if nr else 0
        self.ncb = -(-nc // bsc) if nc else 0
        self.thresh = thresh
        if dense is not None:
            self.copy_from_input_matrix(dense)

    @classmethod
    def from_dense(cls, a, bsr, bsc, thresh, pool=None, ctx=None):
        """BlockSparseMatrix(const Matrix&, bsr, bsc, thresh) blocksparsematrix.hpp:27-32"""
        return cls(a.shape[0], a.shape[1], bsr, bsc, thresh, pool=pool, ctx=ctx, dense=a)

    def __del__(self):
        try:
            lib.bsg_bsm_destroy(self.h)
        except Exception:
            pass

    @property
    def nblocks(self):
        return self.nrb * self.ncb

    def mem_pool(self):
        h = C.c_void_p()
        check(lib.bsg_bsm_pool(self.h, C.byref(h)))
        return BlockMemoryPool(0, ctx=self.ctx, _handle=h)

    def assign(self, other):
        """operator= (occ_ri_k_step.cpp:112)"""
        check(lib.bsg_bsm_assign(self.h, other.h))
        return self

    def copy_from_input_matrix(self, a):
        assert tuple(a.shape) == (self.nr, self.nc), "copy_from_input_matrix: shape mismatch"
        p, where, keep = _buf(a)
        check(lib.bsg_bsm_copy_from_dense(self.h, p, where))
        del keep

    copy_from_input_array = copy_from_input_matrix

    def fill_with_values(self, v):
        check(lib.bsg_bsm_fill(self.h, float(v)))

    def zero(self):
        check(lib.bsg_bsm_zero(self.h))

    def scale(self, s):
        check(lib.bsg_bsm_scale(self.h, float(s)))

    def __imul__(self, s):
        self.scale(s)
        return self

    def __iadd__(self, o):
        check(lib.bsg_bsm_add(self.h, o.h))
        return self

    def __isub__(self, o):
        check(lib.bsg_bsm_sub(self.h, o.h))
        return self

    def add_transpose(self, o):
        check(lib.bsg_bsm_add_transpose(self.h, o.h))

    def calc_frobenius_norms(self):
        check(lib.bsg_bsm_calc_norms(self.h))

    def recompress(self):
        check(lib.bsg_bsm_recompress(self.h))

    def frobenius_norm(self):
        v = C.c_double()
        check(lib.bsg_bsm_frobenius_norm(self.h, C.byref(v)))
        return v.value

    def no_of_alloc_blocks(self):
        v = C.c_size_t()
        check(lib.bsg_bsm_no_of_alloc_blocks(self.h, C.byref(v)))
        return v.value

    def calc_alloc_dim(self):
        v = C.c_size_t()
        check(lib.bsg_bsm_calc_alloc_dim(self.h, C.byref(v)))
        return v.value

    def to_matrix(self, out=None):
        """to_matrix / to_pointer (absent blocks read as zero)"""
        if out is None:
            out = np.zeros((self.nr, self.nc), dtype=np.float64, order="F")
        p, where, keep = _buf(out)
        check(lib.bsg_bsm_to_dense(self.h, p, where))
        if where == BSG_HOST and keep is not out:
            out[...] = keep
        return out

    def mask(self):
        m = np.zeros(self.nblocks, dtype=np.uint8)
        check(lib.bsg_bsm_get_mask(self.h, m.ctypes.data_as(C.c_void_p)))
        return m

    def norms(self):
        n = np.zeros(self.nblocks, dtype=np.float64)
        check(lib.bsg_bsm_get_norms(self.h, n.ctypes.data_as(C.c_void_p)))
        return n


def matmult(C_, A, tA, B, tB, thresh, alpha=1.0, beta=0.0, form=FORM_FP64, n_digits=4):
    """matmult(C, A, transA, B, transB, thresh, alpha, beta); returns the
    number of surviving block products."""
    n = C.c_uint64()
    check(lib.bsg_matmult_form(C_.h, A.h, int(bool(tA)), B.h, int(bool(tB)), float(thresh), float(alpha), float(beta),
                               form, n_digits, C.byref(n)))
    return n.value


def dot(A, B, thresh=0.0):
    v = C.c_double()
    check(lib.bsg_dot(A.h, B.h, float(thresh), C.byref(v)))
    return v.value


def matmult_strassen_dryrun(A, B, thresh_per_block):
    """Decision tree per level (bool arrays, index si + sj*n + sk*n*n) and the
    flop count per level."""
    nb = A.nrb
    sizes = []
    l = 0
    while 2 ** l <= 2 * nb + 1 and l < 64:
        sizes.append((-(-nb // 2 ** (l + 1))) ** 3)
        l += 1
    cap = sum(sizes) + 8
    tree = np.zeros(cap, dtype=np.uint8)
    flops = np.zeros(70, dtype=np.uint64)
    nl = C.c_int()
    check(lib.bsg_strassen_dryrun(A.h, B.h, float(thresh_per_block), C.byref(nl), tree.ctypes.data_as(C.c_void_p),
                                  cap, flops.ctypes.data_as(C.POINTER(C.c_uint64))))
    levels, off = [], 0
    for lv in range(nl.value):
        n = -(-nb // 2 ** (lv + 1))
        levels.append(tree[off:off + n ** 3].astype(bool))
        off += n ** 3
    return levels, flops[: nl.value + 1].copy()


def matmult_strassen_sparse(C_, A, tA, B, tB, thresh, alpha, beta, min_size_for_strassen, form=FORM_FP64,
                            n_digits=4):
    if form == FORM_FP64:
        check(lib.bsg_matmult_strassen_sparse(C_.h, A.h, int(bool(tA)), B.h, int(bool(tB)), float(thresh),
                                              float(alpha), float(beta), int(min_size_for_strassen)))
    else:
        if tA or tB or alpha != 1.0:
            raise BsgError(2, "matmult_strassen_sparse supports no transposes and alpha = 1")
        check(lib.bsg_matmult_strassen_sparse_form(C_.h, A.h, B.h, float(thresh), int(min_size_for_strassen), form,
                                                   n_digits))


def matmult_batched(Cs, As, Bs, thresh, alpha=1.0, beta=0.0, form=FORM_FP64, n_digits=0):
    """C_i = alpha A_i B_i + beta C_i for every i (matmult semantics, no
    transposes); the mixed form runs the tiles of every block-size group in
    one persistent tensor-core launch (up to 8 groups per launch).  Returns
    the surviving block triples of all products."""
    assert len(Cs) == len(As) == len(Bs)
    n = C.c_uint64()
    check(lib.bsg_matmult_batched(len(Cs), _handles(Cs), _handles(As), _handles(Bs), float(thresh), float(alpha),
                                  float(beta), form, int(n_digits), C.byref(n)))
    return n.value


class BatchPlan:
    """A mixed-form batch C_i = alpha A_i B_i captured as a CUDA graph (see
    bsg_batched_plan_create); run() replays it."""

    def __init__(self, Cs, As, Bs, thresh, alpha=1.0, n_digits=0):
        self._keep = (list(Cs), list(As), list(Bs))
        h = C.c_void_p()
        check(lib.bsg_batched_plan_create(len(Cs), _handles(Cs), _handles(As), _handles(Bs), float(thresh),
                                          float(alpha), int(n_digits), C.byref(h)))
        self.h = h

    def run(self):
        check(lib.bsg_batched_plan_run(self.h))

    def __del__(self):
        h = getattr(self, "h", None)
        if h and lib is not None:
            lib.bsg_batched_plan_destroy(h)
            self.h = None


class StrassenScheduler:
    """The learned node scheduler of the hybrid recursion (a 2 x 64 MLP on the
    device scoring Strassen depths and the dense tile against the sparse
    recursion; forward, backward and Adam are the library's own kernels)."""

    def __init__(self, ctx=None, seed=None):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        check(lib.bsg_sched_create(self.ctx.h, C.byref(h)))
        self.h = h
        n = C.c_int()
        check(lib.bsg_sched_param_count(C.byref(n)))
        self.n_params = n.value
        if seed is not None:
            check(lib.bsg_sched_init(self.h, int(seed)))

    def __del__(self):
        h = getattr(self, "h", None)
        if h and lib is not None:
            lib.bsg_sched_destroy(h)
            self.h = None

    @property
    def params(self):
        out = np.empty(self.n_params, np.float32)
        check(lib.bsg_sched_get_params(self.h, out.ctypes.data))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        check(lib.bsg_sched_set_params(self.h, p.ctypes.data))

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, SCHED_FEATURES)
        y = np.empty(len(X), np.float32)
        check(lib.bsg_sched_predict(self.h, X.ctypes.data, len(X), y.ctypes.data))
        return y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, SCHED_FEATURES)
        T = np.ascontiguousarray(T, np.float32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float()
        check(lib.bsg_sched_loss_grad(self.h, X.ctypes.data, T.ctypes.data, len(X), C.byref(loss), g.ctypes.data))
        return float(loss.value), g

    def train(self, X, T, epochs=200, batch=32, lr=3e-3, seed=7):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, SCHED_FEATURES)
        T = np.ascontiguousarray(T, np.float32)
        loss = C.c_float()
        check(lib.bsg_sched_train(self.h, X.ctypes.data, T.ctypes.data, len(X), int(epochs), int(batch), float(lr),
                                  int(seed), C.byref(loss)))
        return float(loss.value)


def strassen_root_features(C_, A, B, thresh):
    """node features of the root node of C = A B's Strassen decision tree and
    whether it may run Strassen or a dense tile (all blocks present, not an
    edge node)"""
    f = np.empty(SCHED_NODE_FEATURES, np.float32)
    ok = C.c_int()
    check(lib.bsg_strassen_root_features(C_.h, A.h, B.h, float(thresh), f.ctypes.data, C.byref(ok)))
    return f, bool(ok.value)


def option_rows(features, options=None):
    """network inputs: node features followed by the one-hot of an option
    (0..2 Strassen depth 1..3, 3 dense tile); one row per (node, option)"""
    F = np.asarray(features, np.float32).reshape(-1, SCHED_NODE_FEATURES)
    opts = np.asarray(range(SCHED_OPTIONS) if options is None else options, np.int64)
    X = np.zeros((len(F) * len(opts), SCHED_FEATURES), np.float32)
    X[:, :SCHED_NODE_FEATURES] = np.repeat(F, len(opts), axis=0)
    X[np.arange(len(X)), SCHED_NODE_FEATURES + np.tile(opts, len(F))] = 1.0
    return X


def matmult_strassen_sparse_sched(C_, A, B, thresh, min_size_for_strassen, policy=SCHED_COST, sched=None,
                                  form=FORM_FP64, n_digits=4):
    """matmult_strassen_sparse with a scheduling policy (SCHED_COST, _NONE,
    _ROOT, _DENSE, _MLP); returns the number of nodes that ran Strassen or a
    dense tile"""
    n = C.c_uint64()
    check(lib.bsg_matmult_strassen_sparse_sched(C_.h, A.h, B.h, float(thresh), int(min_size_for_strassen), form,
                                                int(n_digits), int(policy), sched.h if sched is not None else None,
                                                C.byref(n)))
    return n.value


def _handles(ms):
    arr = (C.c_void_p * len(ms))(*[m.h.value for m in ms])
    return arr


def tensormult_contract(C_, As, tA, Bs, tB, thresh, alpha=1.0, beta=0.0):
    """C_ij = sum_l sum_k op(A^l)_ik op(B^l)_kj"""
    assert len(As) == len(Bs) and len(As) > 0
    check(lib.bsg_tensormult_contract(C_.h, _handles(As), int(bool(tA)), _handles(Bs), int(bool(tB)), len(As),
                                      float(thresh), float(alpha), float(beta)))


def tensormult_batched(Cs, A, tA, Bs, tB, thresh, alpha=1.0, beta=0.0):
    """C^l_ij = sum_k op(A)_ik op(B^l)_kj for every slice l"""
    assert len(Cs) == len(Bs) and len(Bs) > 0
    check(lib.bsg_tensormult_batched(_handles(Cs), A.h, int(bool(tA)), _handles(Bs), int(bool(tB)), len(Bs),
                                     float(thresh), float(alpha), float(beta)))


def rik_occ_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1, form=FORM_FP64, n_digits=4,
                 p_chunk=0, out=None, ctx=None, stats=False, trace=False):
    """K_{mu j} = sum_{P,i} (mu i|P)[(ij|P)+(ji|P)] (occ_ri_k_step.cpp:83-130).

    ints: n_vec2 x n_aux, keys: n_vec2 uint64, c_occ: n_bf x n_occ; numpy
    (host) or torch CUDA tensors (device, all three alike).  trace=True also
    returns the screening state of every aux function (a dict of numpy
    arrays, see bsg_rik_screen_trace): (K, stats, trace)."""
    if trace:
        ctx = ctx or default_context()
        pi, w1, k1 = _buf(ints)
        pk, w2, k2 = _buf(keys, np.uint64)
        pc, w3, k3 = _buf(c_occ)
        if not (w1 == w2 == w3):
            raise BsgError(1, "ints, keys and c_occ must all be host or all device arrays")
        a = RikArgs(n_bf, n_aux, n_occ, ints.shape[0], pi, pk, pc, w1, bs, float(thresh), n_part, form, n_digits,
                    p_chunk)
        if out is None:
            out = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
        po, wo, ko = _buf(out)
        nb, nob = -(-n_bf // bs), -(-n_occ // bs)
        tr = {"mui_norm": np.zeros((n_aux, nob, nb)), "mui_flag": np.zeros((n_aux, nob, nb), np.uint8),
              "ij_flag": np.zeros((n_aux, nob, nob), np.uint8), "ijs_norm": np.zeros((n_aux, nob, nob)),
              "ijs_flag": np.zeros((n_aux, nob, nob), np.uint8), "c_norm": np.zeros((nob, nb))}
        t = ScreenTrace(*[C.c_void_p(tr[k].ctypes.data) for k in
                          ("mui_norm", "mui_flag", "ij_flag", "ijs_norm", "ijs_flag", "c_norm")])
        st = (C.c_uint64 * 5)()
        check(lib.bsg_rik_occ_step_trace(ctx.h, C.byref(a), po, wo, st, C.byref(t)))
        if wo == BSG_HOST and ko is not out:
            out[...] = ko
        del k1, k2, k3
        # [P][jb][a] storage order -> arrays indexed [P, a, jb] (mui) and [P, ib, jb] (ij, ijs), C [a, jb]
        tr = {k: (np.swapaxes(v, -1, -2) if v.ndim >= 2 else v) for k, v in tr.items()}
        tr.update(n_bf=n_bf, n_occ=n_occ, bs=bs, thresh=float(thresh))
        return out, list(st), tr
    ctx = ctx or default_context()
    pi, w1, k1 = _buf(ints)
    pk, w2, k2 = _buf(keys, np.uint64)
    pc, w3, k3 = _buf(c_occ)
    if not (w1 == w2 == w3):
        raise BsgError(1, "ints, keys and c_occ must all be host or all device arrays")
    n_vec2 = ints.shape[0]
    a = RikArgs(n_bf, n_aux, n_occ, n_vec2, pi, pk, pc, w1, bs, float(thresh), n_part, form, n_digits, p_chunk)
    if out is None:
        out = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
    po, wo, ko = _buf(out)
    st = (C.c_uint64 * 5)()
    check(lib.bsg_rik_occ_step(ctx.h, C.byref(a), po, wo, st))
    if wo == BSG_HOST and ko is not out:
        out[...] = ko
    del k1, k2, k3
    return (out, list(st)) if stats else out


def rik_kmn_step(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part=1, form=FORM_FP64, n_digits=4,
                 p_chunk=0, out=None, k_out=False, ctx=None, stats=False):
    """Symmetric K_mn = sum_{P,i} mui_P(m,i) mui_P(n,i) on the occ step's
    screened mui_P (occ_ri_k_step.cpp:102-108), n_bf x n_bf.

    Inputs as rik_occ_step.  k_out=True also returns the occ step's K
    (n_bf x n_occ) from the same pass: (Kmn, K).  stats=True appends the six
    counters (the occ step's five, then the K_mn block products)."""
    ctx = ctx or default_context()
    pi, w1, k1 = _buf(ints)
    pk, w2, k2 = _buf(keys, np.uint64)
    pc, w3, k3 = _buf(c_occ)
    if not (w1 == w2 == w3):
        raise BsgError(1, "ints, keys and c_occ must all be host or all device arrays")
    n_vec2 = ints.shape[0]
    a = RikArgs(n_bf, n_aux, n_occ, n_vec2, pi, pk, pc, w1, bs, float(thresh), n_part, form, n_digits, p_chunk)
    if out is None:
        out = np.zeros((n_bf, n_bf), dtype=np.float64, order="F")
    po, wo, ko = _buf(out)
    kq = kk = None
    pq = None
    if k_out:
        if wo == BSG_HOST:
            kq = np.zeros((n_bf, n_occ), dtype=np.float64, order="F")
        else:  # device output: a column-major n_bf x n_occ view
            import torch
            kq = torch.zeros((n_occ, n_bf), dtype=torch.float64, device=out.device).t()
        pq, wq, kk = _buf(kq)
    st = (C.c_uint64 * 6)()
    check(lib.bsg_rik_kmn_step(ctx.h, C.byref(a), po, pq, wo, st))
    if wo == BSG_HOST and ko is not out:
        out[...] = ko
    if k_out and wo == BSG_HOST and kk is not kq:
        kq[...] = kk
    del k1, k2, k3
    res = (out, kq) if k_out else (out,)
    if stats:
        res = res + (list(st),)
    return res[0] if len(res) == 1 else res


def transform_3c2c(ints_3c, v_m12, bs, thresh, form=FORM_FP64, n_digits=4, out=None, ctx=None, stats=False):
    """(mu nu|P)' = sum_Q (mu nu|Q)(Q|P)^{-1/2} (3c_2c_transform.cpp:44-57);
    stats=True: (out, surviving block products)"""
    ctx = ctx or default_context()
    px, w1, k1 = _buf(ints_3c)
    pv, w2, k2 = _buf(v_m12)
    if w1 != w2:
        raise BsgError(1, "inputs must both be host or both device arrays")
    n_vec2, n_aux = ints_3c.shape
    if out is None:
        out = np.zeros((n_vec2, n_aux), dtype=np.float64, order="F")
    po, wo, ko = _buf(out)
    nsig = C.c_uint64()
    check(lib.bsg_3c2c_transform_nsig(ctx.h, n_vec2, n_aux, px, pv, w1, bs, float(thresh), form, n_digits, po, wo,
                                      C.byref(nsig)))
    if wo == BSG_HOST and ko is not out:
        out[...] = ko
    del k1, k2
    return (out, nsig.value) if stats else out

