"""Multi-rank RI-K step: the aux index P is sharded over ranks.

The reference runs P in an OpenMP static loop (occ_ri_k_step.cpp:99) and sums
the threads' partial K in a critical section (:119-122).  Here each rank takes
one contiguous P range with the same static boundaries, computes its partial
K with the library, and one sum all-reduce combines the partials.  With two
ranks the result is bit-identical to the single-process step with n_part = 2
(one addition of the two partials, which commutes).  On a box with one GPU
the benchmark runs replicas instead (one full step per rank).
"""
from __future__ import annotations

import numpy as np


def p_range(n_aux, rank, world):
    """[lo, hi) of rank's aux functions: libgomp's static schedule (the first
    n_aux % world ranks take one more)"""
    q, r = divmod(int(n_aux), int(world))
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def rik_occ_step_sharded(ints, keys, c_occ, n_bf, n_aux, n_occ, bs, thresh, group=None, compute=None, **kw):
    """K = sum over ranks of the rank's partial step on its P range, summed
    with one all-reduce (torch.distributed; NCCL for CUDA tensors, gloo on the
    host).  ints: n_vec2 x n_aux column-major (numpy, or a CUDA tensor view).
    compute(ints_cols, keys, c_occ, n_bf, n_p, n_occ, bs, thresh) defaults to
    the library's step (strassen_gb300.api.rik_occ_step with **kw)."""
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    lo, hi = p_range(n_aux, rank, world)
    cols = ints[:, lo:hi]
    if compute is None:
        from . import api

        part = api.rik_occ_step(cols, keys, c_occ, n_bf, hi - lo, n_occ, bs, thresh, **kw)
    else:
        part = compute(cols, keys, c_occ, n_bf, hi - lo, n_occ, bs, thresh)
    if isinstance(part, np.ndarray):
        t = torch.from_numpy(np.asfortranarray(part).ravel(order="F").copy())
    else:
        t = part.T.contiguous().view(-1)  # column-major order of a (n_bf x n_occ) view
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    if isinstance(part, np.ndarray):
        return t.numpy().reshape((n_bf, n_occ), order="F")
    return t.view(n_occ, n_bf).T
