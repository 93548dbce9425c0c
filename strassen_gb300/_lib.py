"""ctypes binding of libbsgpu.so (the C ABI declared in include/bsgpu.h).

The library is the product path; there is no fallback.  If the shared
library is missing this module raises at import time.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbsgpu.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is not built; run `python -m strassen_gb300.build` (or __graft_entry__.build())")

lib = C.CDLL(LIB_PATH)

c_size = C.c_size_t
c_dbl = C.c_double
c_int = C.c_int
c_vp = C.c_void_p
c_u64p = C.POINTER(C.c_uint64)

BSG_HOST, BSG_DEVICE = 0, 1
FORM_FP64, FORM_OZAKI = 0, 1
ERRORS = {1: "BSG_ERR_ARG", 2: "BSG_ERR_PRECOND", 3: "BSG_ERR_CUDA", 4: "BSG_ERR_NOMEM", 5: "BSG_ERR_TIMEOUT",
          6: "BSG_ERR_UNSUPPORTED"}


class BsgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RikArgs(C.Structure):
    _fields_ = [("n_bf", c_size), ("n_aux", c_size), ("n_occ", c_size), ("n_vec2", c_size), ("ints", c_vp),
                ("keys", c_vp), ("c_occ", c_vp), ("where", c_int), ("bs", c_size), ("thresh", c_dbl),
                ("n_part", c_int), ("form", c_int), ("n_digits", c_int), ("p_chunk", c_size)]


class ScreenTrace(C.Structure):
    _fields_ = [("mui_norm", c_vp), ("mui_flag", c_vp), ("ij_flag", c_vp), ("ijs_norm", c_vp), ("ijs_flag", c_vp),
                ("c_norm", c_vp)]


def _sig(name, args, res=c_int):
    f = getattr(lib, name)
    f.argtypes = args
    f.restype = res
    return f


_sig("bsg_last_error", [], C.c_char_p)
_sig("bsg_version", [])
_sig("bsg_ctx_create", [c_int, c_vp, C.POINTER(c_vp)])
_sig("bsg_ctx_destroy", [c_vp])
_sig("bsg_ctx_sync", [c_vp])
_sig("bsg_ctx_launch_count", [c_vp, c_u64p])
_sig("bsg_ctx_set_timing", [c_vp, c_int])
_sig("bsg_ctx_gemm_timing", [c_vp, c_u64p, C.POINTER(c_dbl), C.POINTER(c_dbl)])
_sig("bsg_ctx_gemm_stalls", [c_vp, c_u64p])
_sig("bsg_rik_occ_step_noalloc", [C.POINTER(RikArgs), c_vp, c_vp, c_u64p])
_sig("bsg_pool_create", [c_vp, c_size, C.POINTER(c_vp)])
_sig("bsg_pool_release", [c_vp])
_sig("bsg_pool_adjust_blocksize", [c_vp, c_size])
_sig("bsg_pool_release_all_memory", [c_vp])
_sig("bsg_pool_stats", [c_vp, C.POINTER(c_size), C.POINTER(c_size), C.POINTER(c_size)])
_sig("bsg_bsm_create", [c_vp, c_size, c_size, c_size, c_size, c_dbl, c_vp, C.POINTER(c_vp)])
_sig("bsg_bsm_destroy", [c_vp])
_sig("bsg_bsm_info", [c_vp, c_vp, C.POINTER(c_dbl)])
_sig("bsg_bsm_pool", [c_vp, C.POINTER(c_vp)])
_sig("bsg_bsm_assign", [c_vp, c_vp])
_sig("bsg_bsm_copy_from_dense", [c_vp, c_vp, c_int])
_sig("bsg_bsm_fill", [c_vp, c_dbl])
_sig("bsg_bsm_zero", [c_vp])
_sig("bsg_bsm_scale", [c_vp, c_dbl])
_sig("bsg_bsm_add", [c_vp, c_vp])
_sig("bsg_bsm_sub", [c_vp, c_vp])
_sig("bsg_bsm_add_transpose", [c_vp, c_vp])
_sig("bsg_bsm_calc_norms", [c_vp])
_sig("bsg_bsm_recompress", [c_vp])
_sig("bsg_bsm_frobenius_norm", [c_vp, C.POINTER(c_dbl)])
_sig("bsg_bsm_no_of_alloc_blocks", [c_vp, C.POINTER(c_size)])
_sig("bsg_bsm_calc_alloc_dim", [c_vp, C.POINTER(c_size)])
_sig("bsg_bsm_to_dense", [c_vp, c_vp, c_int])
_sig("bsg_bsm_get_mask", [c_vp, c_vp])
_sig("bsg_bsm_get_norms", [c_vp, c_vp])
_sig("bsg_dot", [c_vp, c_vp, c_dbl, C.POINTER(c_dbl)])
_sig("bsg_matmult", [c_vp, c_vp, c_int, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_u64p])
_sig("bsg_matmult_form", [c_vp, c_vp, c_int, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_int, c_int, c_u64p])
_sig("bsg_strassen_dryrun", [c_vp, c_vp, c_dbl, C.POINTER(c_int), c_vp, c_size, c_u64p])
_sig("bsg_matmult_strassen_sparse", [c_vp, c_vp, c_int, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_size])
_sig("bsg_matmult_strassen_sparse_form", [c_vp, c_vp, c_vp, c_dbl, c_size, c_int, c_int])
_sig("bsg_tensormult_contract", [c_vp, c_vp, c_int, c_vp, c_int, c_size, c_dbl, c_dbl, c_dbl])
_sig("bsg_tensormult_batched", [c_vp, c_vp, c_int, c_vp, c_int, c_size, c_dbl, c_dbl, c_dbl])
_sig("bsg_rik_occ_step", [c_vp, C.POINTER(RikArgs), c_vp, c_int, c_u64p])
_sig("bsg_rik_occ_step_trace", [c_vp, C.POINTER(RikArgs), c_vp, c_int, c_u64p, C.POINTER(ScreenTrace)])
_sig("bsg_rik_kmn_step", [c_vp, C.POINTER(RikArgs), c_vp, c_vp, c_int, c_u64p])
_sig("bsg_3c2c_transform", [c_vp, c_size, c_size, c_vp, c_vp, c_int, c_size, c_dbl, c_int, c_int, c_vp, c_int])
_sig("bsg_3c2c_transform_nsig", [c_vp, c_size, c_size, c_vp, c_vp, c_int, c_size, c_dbl, c_int, c_int, c_vp, c_int,
                                 c_u64p])
c_flt = C.c_float
_sig("bsg_sched_create", [c_vp, C.POINTER(c_vp)])
_sig("bsg_sched_destroy", [c_vp])
_sig("bsg_sched_param_count", [C.POINTER(c_int)])
_sig("bsg_sched_init", [c_vp, C.c_uint64])
_sig("bsg_sched_set_params", [c_vp, c_vp])
_sig("bsg_sched_get_params", [c_vp, c_vp])
_sig("bsg_sched_predict", [c_vp, c_vp, c_int, c_vp])
_sig("bsg_sched_loss_grad", [c_vp, c_vp, c_vp, c_int, C.POINTER(c_flt), c_vp])
_sig("bsg_sched_train", [c_vp, c_vp, c_vp, c_int, c_int, c_int, c_flt, C.c_uint64, C.POINTER(c_flt)])
_sig("bsg_strassen_root_features", [c_vp, c_vp, c_vp, c_dbl, c_vp, C.POINTER(c_int)])
_sig("bsg_matmult_strassen_sparse_sched", [c_vp, c_vp, c_vp, c_dbl, c_size, c_int, c_int, c_int, c_vp, c_u64p])

_sig("bsg_matmult_batched", [c_size, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_dbl, c_int, c_int, c_u64p])
_sig("bsg_batched_plan_create", [c_size, c_vp, c_vp, c_vp, c_dbl, c_dbl, c_int, C.POINTER(c_vp)])
_sig("bsg_batched_plan_run", [c_vp])
_sig("bsg_batched_plan_destroy", [c_vp])
_sig("bsg_ctx_set_autotune", [c_vp, c_int])
_sig("bsg_ctx_autotune_entries", [c_vp, c_vp, c_int, C.POINTER(c_int)])

SCHED_COST, SCHED_NONE, SCHED_ROOT, SCHED_MLP, SCHED_DENSE = 0, 1, 2, 3, 4
SCHED_NODE_FEATURES, SCHED_OPTIONS = 25, 4
SCHED_FEATURES = SCHED_NODE_FEATURES + SCHED_OPTIONS


def check(status):
    if status != 0:
        raise BsgError(status, lib.bsg_last_error().decode(errors="replace"))
