"""Multi-rank RI-K on CPU: two gloo ranks, each runs its P range (libgomp's
static boundaries) and one all-reduce sums the partial K -- bit-identical to
the single-process step with n_part = 2.  The oracle stands in for the
per-rank device step (the host-side sharding logic is what is tested)."""
import os
import socket

import numpy as np
import pytest

from strassen_gb300.shard import p_range


def test_p_range_is_libgomp_static():
    for n in (0, 1, 7, 113, 3360):
        for w in (1, 2, 3, 8):
            rs = [p_range(n, r, w) for r in range(w)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(rs[i][1] == rs[i + 1][0] for i in range(w - 1))
            sizes = [hi - lo for lo, hi in rs]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, inputs, out_dir):
    import torch.distributed as dist

    from oracle import oracle as O
    from strassen_gb300.shard import rik_occ_step_sharded

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ints, keys, C, n_bf, n_aux, n_occ, bs, thr = inputs
    K = rik_occ_step_sharded(ints, keys, C, n_bf, n_aux, n_occ, bs, thr,
                             compute=lambda *a: O.rik_occ_step(*a, n_part=1))
    np.save(os.path.join(out_dir, f"K{rank}.npy"), K)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("system", ["h2o", "synthetic"])
def test_two_rank_rik_matches_single_process(tmp_path, h2o, system, oracle):
    import torch.multiprocessing as mp

    from strassen_gb300 import synth as S

    if system == "h2o":
        ints, keys, C, n_bf, n_aux, n_occ = (h2o["ints"], h2o["keys"], h2o["c"], h2o["n_bf"], h2o["n_aux"],
                                             h2o["n_occ"])
        bs, thr = 3, 1e-20
    else:
        s = S.RikSystem(seed=5, n_atoms=6, nbf=8, naux=20, n_occ=12, box=6.0)
        ints, keys, C, n_bf, n_aux, n_occ = s.ints_3c(), s.keys, s.c_occ(), s.n_bf, s.n_aux, s.n_occ
        bs, thr = 8, 1e-10
    inputs = (np.asfortranarray(ints), np.ascontiguousarray(keys), np.asfortranarray(C), n_bf, n_aux, n_occ, bs, thr)
    mp.start_processes(_rank_main, args=(2, _free_port(), inputs, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    K0 = np.load(tmp_path / "K0.npy")
    K1 = np.load(tmp_path / "K1.npy")
    ref = oracle.rik_occ_step(ints, keys, C, n_bf, n_aux, n_occ, bs, thr, n_part=2)
    assert np.array_equal(K0.view(np.uint64), ref.view(np.uint64))
    assert np.array_equal(K1.view(np.uint64), ref.view(np.uint64))
