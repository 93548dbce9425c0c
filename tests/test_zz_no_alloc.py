"""The allocation-free RI-K entry point (bsg_rik_occ_step_noalloc).

It exists for callers that cannot allocate device memory themselves -- code
under a framework whose caching allocator owns the device heap, processes
with a fixed memory budget, streams that cannot absorb cudaFree's implicit
synchronization -- and keeps every intermediate in a fixed 32 MiB device
array inside the library.  These tests call it through the C ABI twice in a
row (the array keeps the previous call's contents, which must not leak into
the next result) and compare with bsg_rik_occ_step, bit for bit.  This file
is collected last so that a run stopping at the first failure has run every
other test already; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from strassen_gb300 import synth as S
from tests.conftest import same_bits

pytestmark = pytest.mark.gpu


def _noalloc(api, ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, n_part, p_chunk=0, stream=None, stats=True):
    """one call through the C ABI; stream: a torch.cuda.Stream (None: the
    legacy default stream); stats False passes stats_out = NULL, with which
    the call only enqueues its kernels"""
    import torch

    K = torch.zeros((n_occ, n_bf), dtype=torch.float64, device="cuda").T  # column-major n_bf x n_occ
    a = api.RikArgs(n_bf, n_aux, n_occ, ints.shape[0], C.c_void_p(ints.data_ptr()), C.c_void_p(keys.data_ptr()),
                    C.c_void_p(c_occ.data_ptr()), api.BSG_DEVICE, bs, float(thresh), n_part, api.FORM_FP64, 0, p_chunk)
    fn = api.lib.bsg_rik_occ_step_noalloc
    fn.argtypes = [C.POINTER(api.RikArgs), C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]
    fn.restype = C.c_int
    torch.cuda.synchronize()
    st = (C.c_uint64 * 5)()
    h = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = fn(C.byref(a), C.c_void_p(K.data_ptr()), h, st if stats else None)
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return rc, K.cpu().numpy(), list(st)


def _dev(a, dtype=None):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()
    return t.T if t.dim() == 2 else t


def _case(api, ctx, ints, keys, c, n_bf, n_aux, n_occ, bs, thr, n_part, p_chunk=0):
    di, dk, dc = _dev(ints), _dev(keys.view(np.int64)), _dev(c)
    K_ref, st_ref = api.rik_occ_step(di, dk, dc, n_bf, n_aux, n_occ, bs, thr, n_part=n_part, ctx=ctx, stats=True)
    K_ref = np.asarray(K_ref)
    for _ in range(2):  # two calls in a row share the scratch array
        rc, K, st = _noalloc(api, di, dk, dc, n_bf, n_aux, n_occ, bs, thr, n_part, p_chunk)
        assert rc == 0, api.lib.bsg_last_error()
        assert same_bits(K, K_ref)
        assert st[:3] == st_ref[:3]


@pytest.mark.parametrize("n_part", [1, 4])
def test_noalloc_h2o(api, ctx, h2o, n_part):
    d = h2o
    _case(api, ctx, d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part)
    assert np.linalg.norm(_noalloc(api, _dev(d["ints"]), _dev(d["keys"].view(np.int64)), _dev(d["c"]), d["n_bf"],
                                   d["n_aux"], d["n_occ"], 3, 1e-20, n_part)[1]) == pytest.approx(10.415071322740426,
                                                                                                  rel=1e-14)


def test_noalloc_synthetic_chunked(api, oracle, ctx):
    s = S.RikSystem(seed=9, n_atoms=5, nbf=24, naux=12, n_occ=20, box=8.0)
    B = oracle.transform_3c2c(s.ints_3c(), s.v_m12(), 24, 1e-10)
    for p_chunk in (0, 7):
        _case(api, ctx, B, s.keys, s.c_occ(), s.n_bf, s.n_aux, s.n_occ, 24, 1e-10, 3, p_chunk)


def test_noalloc_rejects_oversize(api):
    import torch

    n_bf, n_occ, n_vec2 = 4096, 8, 4  # one aux function needs 4096^2 doubles > 32 MiB
    ints = torch.zeros((1, n_vec2), dtype=torch.float64, device="cuda").T
    keys = torch.zeros(n_vec2, dtype=torch.int64, device="cuda")
    c = torch.zeros((n_occ, n_bf), dtype=torch.float64, device="cuda").T
    rc, _, _ = _noalloc(api, ints, keys, c, n_bf, 1, n_occ, 32, 1e-10, 1)
    assert rc == 1 and b"32 MiB" in api.lib.bsg_last_error()


def test_noalloc_on_a_stream_without_stats(api, ctx, h2o):
    """on a non-default stream, stats_out NULL (the call only enqueues work):
    the same bits, twice in a row"""
    import torch

    d = h2o
    di, dk, dc = _dev(d["ints"]), _dev(d["keys"].view(np.int64)), _dev(d["c"])
    K_ref = np.asarray(api.rik_occ_step(di, dk, dc, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, n_part=2, ctx=ctx))
    st = torch.cuda.Stream()
    for _ in range(2):
        rc, K, _ = _noalloc(api, di, dk, dc, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 2, stream=st, stats=False)
        assert rc == 0, api.lib.bsg_last_error()
        assert same_bits(K, K_ref)


def test_noalloc_bad_key(api, ctx, h2o):
    """a key outside the N_bf x N_bf matrix is never written: K is NaN, and a
    call with stats_out also returns BSG_ERR_ARG; the next good call is exact"""
    d = h2o
    keys = d["keys"].copy()
    keys[7] = d["n_bf"] * d["n_bf"]  # one past the matrix
    di, dc = _dev(d["ints"]), _dev(d["c"])
    rc, K, _ = _noalloc(api, di, _dev(keys.view(np.int64)), dc, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 1,
                        stats=False)
    assert rc == 0 and np.isnan(K).all()
    rc, K, _ = _noalloc(api, di, _dev(keys.view(np.int64)), dc, d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 1)
    assert rc == 1 and b"v2m key" in api.lib.bsg_last_error()
    assert np.isnan(K).all()
    _case(api, ctx, d["ints"], d["keys"], d["c"], d["n_bf"], d["n_aux"], d["n_occ"], 3, 1e-20, 1)
