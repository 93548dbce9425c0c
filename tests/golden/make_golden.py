"""Regenerates the golden fixtures in this directory from the reference.

Run where the reference sources are available (they are read from
``$REF_DIR``, default ``/root/reference``); it builds ``oracle/_ref`` first.

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

REF_DIR = os.environ.get("REF_DIR", "/root/reference")
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


def main():
    subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], env=dict(os.environ, REF_DIR=REF_DIR))
    if sys.argv[1:] == ["kmn"]:
        kmn()
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
    print("golden fixtures written; driver norm line", norm_line)


if __name__ == "__main__":
    main()
