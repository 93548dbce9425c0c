"""The reference's drivers rebuilt against the C++ facade, run on the GPU with
the reference's own H2O data files: the printed results match the
reference's known answers."""
import os
import re
import subprocess

import numpy as np
import pytest

from strassen_gb300 import synth as S

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "strassen_gb300", "drivers", "bin")
G = os.path.join(ROOT, "tests", "golden")


def _run(name, *args):
    exe = os.path.join(BIN, name)
    if not os.path.exists(exe):
        from strassen_gb300 import build as B

        B.build_drivers()
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_occ_ri_k_driver_h2o():
    out = _run("occ_ri_k_step", 24, 113, 5, 322, os.path.join(G, "h2o_3c_ints_PQm12.bin"),
               os.path.join(G, "h2o_occ_mo.bin"), os.path.join(G, "h2o_v2m_key.bin"), 3, 1e-20)
    assert "L2 norm of output = 1.041507e+01" in out  # the reference driver's line (test_occ_ri_k_h2o.sh)
    rmsd = [float(x) for x in re.findall(r"relative RMSD = (\S+)", out)]
    assert len(rmsd) == 3 and max(rmsd) < 1e-9


def test_3c2c_driver_h2o():
    out = _run("3c_2c_transform", 24, 113, 322, os.path.join(G, "h2o_3c_ints.bin"), os.path.join(G, "h2o_2c_inv05.bin"),
               3, 1e-20)
    ref = np.fromfile(os.path.join(G, "h2o_3c_ints_PQm12.bin"))  # the reference's transformed integrals
    norm = float(re.search(r"L2 norm of output = (\S+)", out).group(1))
    assert abs(norm - np.linalg.norm(ref)) <= 1e-6 * np.linalg.norm(ref)
    assert float(re.search(r"relative RMSD = (\S+)", out).group(1)) < 1e-10


def test_strassen_driver(tmp_path):
    n, bs = 512, 64
    a = S.decay_matrix(8, 1, n, n, bs, 6.0)
    b = S.decay_matrix(8, 2, n, n, bs, 6.0)
    fa, fb = tmp_path / "a.bin", tmp_path / "b.bin"
    np.asfortranarray(a).T.tofile(fa)  # column-major raw doubles, the reference's format
    np.asfortranarray(b).T.tofile(fb)
    out = _run("strassen", bs, 256, 1e-10, 2, n, fa, fb)
    rmsd = [float(x) for x in re.findall(r"relative RMSD = (\S+)", out)]
    assert len(rmsd) == 4 and max(rmsd) < 1e-8
