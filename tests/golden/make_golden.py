"""Regenerates the golden fixtures in this directory from the reference.

Run where the reference sources are available (they are read from
``$REF_DIR``, default: a checkout named ``reference`` beside this repository);
it builds ``oracle/_ref`` first.

* ``h2o_*.bin``  -- the reference's own H2O inputs, copied byte for byte
  (raw little-endian column-major, the format of matrix.hpp:200-227).
* ``h2o_golden.npz`` -- outputs of the compiled reference on them: the
  occ-RI-K K matrix (occ_ri_k_step.cpp:83-130, partitions 1 and 4) and the
  3c->2c transform (3c_2c_transform.cpp:44-57), plus the norm line printed by
  the reference's own driver binary.
* ``h2o_kmn_golden.npz`` -- the symmetric exchange matrix K_mn =
  sum_{P,i} mui_P(m,i) mui_P(n,i) built on the compiled reference's classes
  (its mui_P, occ_ri_k_step.cpp:102-108, then matmult(Ks, mui, N, mui, T)),
  partitions 1 and 4, thresholds 1e-20 and 1e-6.  ``make_golden.py kmn``
  rewrites only this file.
* ``config1_golden.npz`` -- the compiled reference's screened matmult and
  hybrid Strassen product at the Strassen benchmark's shape (n 2048, block
  64); ``make_golden.py config1`` rewrites only this file.
* ``config4s_golden.npz`` -- the same for the large Strassen shape's envelope
  at n 2048 (dense core, exp(-|I-J|/10) tails, Strassen depth 0..3);
  ``make_golden.py config4s`` rewrites only this file.
* ``ref_cases.npz`` -- small seeded matmult / Strassen / dry-run cases with
  the compiled reference's results, masks and norms (Strassen outputs as
  SHA-256 of their bytes).  Inputs are rebuilt from the stored per-block
  envelopes with strassen_gb300.synth (bit-identical on every host).
"""
import hashlib
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from strassen_gb300 import synth as S  # noqa: E402

REF_DIR = os.environ.get("REF_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
H2O = {
    "h2o_3c_ints.bin": "3c_ints_h2o.data",
    "h2o_3c_ints_PQm12.bin": "3c_ints_PQm12_h2o.data",
    "h2o_2c_inv05.bin": "2c_ints_inv05_h2o.data",
    "h2o_occ_mo.bin": "occ_mo_h2o.data",
    "h2o_v2m_key.bin": "v2m_key_h2o.data",
}
N_BF, N_AUX, N_OCC, N_VEC2, BS = 24, 113, 5, 322, 3


def h2o_inputs():
    ints = np.fromfile(os.path.join(HERE, "h2o_3c_ints_PQm12.bin")).reshape(N_AUX, N_VEC2).T
    c = np.fromfile(os.path.join(HERE, "h2o_occ_mo.bin")).reshape(N_OCC, N_BF).T
    keys = np.fromfile(os.path.join(HERE, "h2o_v2m_key.bin"), dtype=np.uint64)
    return ints, keys, c


def kmn():
    ints, keys, c = h2o_inputs()
    out = {}
    for n_part in (1, 4):
        for tag, thr in (("t20", 1e-20), ("t6", 1e-6)):
            out[f"Kmn_part{n_part}_{tag}"] = O.ref_rik_kmn_step(ints, keys, c, N_BF, N_AUX, N_OCC, BS, thr, n_part)
    np.savez(os.path.join(HERE, "h2o_kmn_golden.npz"), **out)


# The Strassen benchmark shape (n 2048, block 64, blocks scaled by
# exp(-|I-J|/6), inputs stored at threshold 0 as main.cpp stores them,
# products screened at 1e-10, one Winograd level: min_size_for_strassen 1024)
CFG1 = dict(n=2048, bs=64, L=6.0, seed=1, thresh=1e-10, min_size=1024)


def config1_env():
    """per-block envelope exp(-|I-J|/L); stored in the fixture, because exp
    may round differently in the last place on another host"""
    c = CFG1
    return S.decay_env(c["n"] // c["bs"], c["n"] // c["bs"], c["L"])


def config1_inputs(env=None):
    c = CFG1
    env = config1_env() if env is None else env
    A = S.from_block_env(c["seed"], 1, c["n"], c["n"], c["bs"], env)
    B = S.from_block_env(c["seed"], 2, c["n"], c["n"], c["bs"], env)
    return A, B


def config1():
    """config1_golden.npz: the compiled reference's screened matmult (C = A B,
    beta 0: output, block mask and cached norms) and matmult_strassen_sparse
    (C pre-filled with zeros) at the benchmark shape, outputs as SHA-256 of
    their bytes, plus the dry-run tree and the surviving-pair count of the
    oracle (the reference's matmult does not report it)."""
    c = CFG1
    env = config1_env()
    A, B = config1_inputs(env)
    bs, thr = c["bs"], c["thresh"]
    out, mask, norms = O.ref_matmult(A, 0.0, (bs, bs), B, 0.0, (bs, bs), 0, 0, thr, 1.0, 0.0)
    oA, oB = O.OBsm(c["n"], c["n"], bs, bs, 0.0, A), O.OBsm(c["n"], c["n"], bs, bs, 0.0, B)
    oC = O.OBsm(c["n"], c["n"], bs, bs, 0.0)
    nsig = O.matmult(oC, oA, 0, oB, 0, thr)
    assert np.array_equal(oC.to_dense(), out), "oracle and compiled reference differ"
    st = O.ref_strassen(A, B, bs, 0.0, thr, c["min_size"])
    levels = O.ref_dryrun(A, B, bs, 0.0, thr * bs ** 3)
    dense = A @ B
    sha = lambda x: np.array(hashlib.sha256(np.asfortranarray(x).tobytes(order="F")).hexdigest())
    np.savez_compressed(os.path.join(HERE, "config1_golden.npz"), params=np.array([c["n"], bs, c["L"], c["seed"], thr,
                                                                                  c["min_size"]]),
                        env=env, mm_sha256=sha(out), mm_mask=mask, mm_norms=norms, mm_nsig=np.array(nsig),
                        mm_fro=np.array(np.linalg.norm(out)), st_sha256=sha(st), st_fro=np.array(np.linalg.norm(st)),
                        tree=np.concatenate(levels) if levels else np.zeros(0, np.uint8),
                        mm_rel_err_dense=np.array(np.linalg.norm(out - dense) / np.linalg.norm(dense)),
                        st_rel_err_dense=np.array(np.linalg.norm(st - dense) / np.linalg.norm(dense)))
    print("config1: nsig", nsig, "rel err vs dense", np.linalg.norm(out - dense) / np.linalg.norm(dense),
          np.linalg.norm(st - dense) / np.linalg.norm(dense))


# The large Strassen shape's envelope at a size the reference finishes in
# seconds: n 2048, block 64, a dense core of the first 512 rows and columns
# (a quarter, as 4096 of 16384), exp(-|I-J|/10) tails, products screened at
# 1e-9, Strassen depth 0..3 (min_size_for_strassen n / 2^depth)
CFG4S = dict(n=2048, bs=64, L=10.0, core=512, seed=4, thresh=1e-9, depths=(0, 1, 2, 3))


def config4s_env():
    """per-block envelope (stored in the fixture, as for config1)"""
    c = CFG4S
    return S.decay_env(c["n"] // c["bs"], c["n"] // c["bs"], c["L"], c["core"] // c["bs"])


def config4s_inputs(env=None):
    c = CFG4S
    env = config4s_env() if env is None else env
    A = S.from_block_env(c["seed"], 1, c["n"], c["n"], c["bs"], env)
    B = S.from_block_env(c["seed"], 2, c["n"], c["n"], c["bs"], env)
    return A, B


def config4s():
    """config4s_golden.npz: the compiled reference's matmult_strassen_sparse
    at each depth (SHA-256 of the output bytes), its dry-run tree, and the
    screened matmult's SHA-256 and surviving-pair count (oracle)."""
    c = CFG4S
    env = config4s_env()
    A, B = config4s_inputs(env)
    bs, thr, n = c["bs"], c["thresh"], c["n"]
    sha = lambda x: np.array(hashlib.sha256(np.asfortranarray(x).tobytes(order="F")).hexdigest())
    out = {"params": np.array([n, bs, c["L"], c["core"], c["seed"], thr]), "env": env}
    mm, _, _ = O.ref_matmult(A, 0.0, (bs, bs), B, 0.0, (bs, bs), 0, 0, thr, 1.0, 0.0)
    oA, oB = O.OBsm(n, n, bs, bs, 0.0, A), O.OBsm(n, n, bs, bs, 0.0, B)
    out["mm_nsig"] = np.array(O.matmult(O.OBsm(n, n, bs, bs, 0.0), oA, 0, oB, 0, thr))
    out["mm_sha256"] = sha(mm)
    levels = O.ref_dryrun(A, B, bs, 0.0, thr * bs ** 3)
    out["tree"] = np.concatenate(levels) if levels else np.zeros(0, np.uint8)
    for d in c["depths"]:
        st = O.ref_strassen(A, B, bs, 0.0, thr, n >> d)
        out[f"st_d{d}_sha256"] = sha(st)
        out[f"st_d{d}_rel_vs_mm"] = np.array(np.linalg.norm(st - mm) / np.linalg.norm(mm))
        print("config4s depth", d, "rel vs matmult", float(out[f"st_d{d}_rel_vs_mm"]))
    np.savez_compressed(os.path.join(HERE, "config4s_golden.npz"), **out)


def main():
    subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], env=dict(os.environ, REF_DIR=REF_DIR))
    if sys.argv[1:] == ["kmn"]:
        kmn()
        return
    if sys.argv[1:] == ["config1"]:
        config1()
        return
    if sys.argv[1:] == ["config4s"]:
        config4s()
        return
    for dst, src in H2O.items():
        shutil.copyfile(os.path.join(REF_DIR, src), os.path.join(HERE, dst))
    ints = np.fromfile(os.path.join(HERE, "h2o_3c_ints_PQm12.bin")).reshape(N_AUX, N_VEC2).T
    x3c = np.fromfile(os.path.join(HERE, "h2o_3c_ints.bin")).reshape(N_AUX, N_VEC2).T
    v = np.fromfile(os.path.join(HERE, "h2o_2c_inv05.bin")).reshape(N_AUX, N_AUX).T
    c = np.fromfile(os.path.join(HERE, "h2o_occ_mo.bin")).reshape(N_OCC, N_BF).T
    keys = np.fromfile(os.path.join(HERE, "h2o_v2m_key.bin"), dtype=np.uint64)
    k1 = O.ref_rik_occ_step(ints, keys, c, N_BF, N_AUX, N_OCC, BS, 1e-20, 1)
    k4 = O.ref_rik_occ_step(ints, keys, c, N_BF, N_AUX, N_OCC, BS, 1e-20, 4)
    # 3c->2c: matmult(out, X_bsm, V_bsm, thresh, 1, 1) on a zero-filled out
    t3, _, _ = O.ref_matmult(x3c, 0.0, (BS, BS), v, 0.0, (BS, BS), 0, 0, 1e-20, 1.0, 1.0, c_mode=1, c_fill=0.0)
    drv = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "occ_ri_k_step"), str(N_BF), str(N_AUX), str(N_OCC),
                          str(N_VEC2), "3c_ints_PQm12_h2o.data", "occ_mo_h2o.data", "v2m_key_h2o.data", str(BS),
                          "1e-20"], cwd=REF_DIR, capture_output=True, text=True, check=True).stdout
    norm_line = re.search(r"L2 norm of output = (\S+)", drv).group(1)
    np.savez(os.path.join(HERE, "h2o_golden.npz"), K_part1=k1, K_part4=k4, X_PQm12=t3,
             driver_norm_line=np.array(norm_line))
    kmn()

    # Small seeded cases.  Inputs are rebuilt in the tests from (seed,
    # stream, per-block envelope table) with strassen_gb300.synth, which is
    # bit-identical on every host; large outputs are stored as SHA-256 of
    # their bytes plus the Frobenius norm.
    rng = np.random.default_rng(20240601)
    cases = {}
    # screened matmult: (m, k, n, bs, tA, tB, alpha, beta, c_mode, thresh)
    mm = [(70, 50, 45, 8, 0, 0, 1.0, 0.0, 0, 1e-9), (70, 50, 45, 8, 1, 0, 1.0, 1.0, 1, 1e-9),
          (64, 64, 64, 16, 0, 1, 0.5, 2.0, 2, 1e-7), (33, 47, 29, 5, 1, 1, 1.0, 0.0, 0, 1e-9),
          (96, 96, 96, 24, 0, 0, 1.0, 1.0, 1, 1e-10), (130, 70, 90, 32, 0, 0, -1.0, 0.0, 0, 1e-8)]
    for i, (m, k, n, bs, tA, tB, al, be, cm, thr) in enumerate(mm):
        ash = (k, m) if tA else (m, k)
        bsh = (n, k) if tB else (k, n)
        envA = np.exp(-rng.uniform(0, 30, size=(-(-ash[0] // bs), -(-ash[1] // bs))))
        envB = np.exp(-rng.uniform(0, 30, size=(-(-bsh[0] // bs), -(-bsh[1] // bs))))
        A = S.from_block_env(7, 3 * i, ash[0], ash[1], bs, envA)
        B = S.from_block_env(7, 3 * i + 1, bsh[0], bsh[1], bs, envB)
        Cin = S.gauss_matrix(7, 3 * i + 2, m, n)
        out, mask, norms = O.ref_matmult(A, 1e-12, (bs, bs), B, 1e-12, (bs, bs), tA, tB, thr, al, be, c_mode=cm,
                                         c_fill=0.0, c_in=Cin, c_thresh=1e-3)
        cases[f"mm{i}_envA"] = envA
        cases[f"mm{i}_envB"] = envB
        cases[f"mm{i}_params"] = np.array([m, k, n, bs, tA, tB, al, be, cm, thr])
        cases[f"mm{i}_out"] = out
        cases[f"mm{i}_mask"] = mask
        cases[f"mm{i}_norms"] = norms
    # Strassen: (n, bs, L, core, thresh, min_size)
    st = [(256, 32, 3.0, 0, 0.0, 64), (384, 32, 2.0, 128, 1e-7, 0), (512, 32, 1.0, 256, 0.0, 128),
          (512, 32, 1.0, 256, 1e-7, 64), (256, 64, 4.0, 0, 1e-9, 128)]
    for i, (n, bs, L, core, thr, ms) in enumerate(st):
        env = S.decay_env(n // bs, n // bs, L, core // bs)
        A = S.from_block_env(11, 2 * i, n, n, bs, env)
        B = S.from_block_env(11, 2 * i + 1, n, n, bs, env)
        out = O.ref_strassen(A, B, bs, 0.0, thr, ms)
        cases[f"st{i}_env"] = env
        cases[f"st{i}_params"] = np.array([n, bs, thr, ms])
        cases[f"st{i}_sha256"] = np.array(hashlib.sha256(np.asfortranarray(out).tobytes(order="F")).hexdigest())
        cases[f"st{i}_fro"] = np.array(np.linalg.norm(out))
        levels = O.ref_dryrun(A, B, bs, 0.0, thr * bs ** 3)
        cases[f"st{i}_tree"] = np.concatenate(levels) if levels else np.zeros(0, np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **cases)
    config1()
    config4s()
    print("golden fixtures written; driver norm line", norm_line)


if __name__ == "__main__":
    main()
