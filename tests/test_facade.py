"""C++ facade (include/bsgpu.hpp): the reference's binary matrix file format
(matrix.hpp:200-227), and the rebuilt drivers' argument handling (no GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")

PROG = r"""
#include <cstdio>
#include "bsgpu.hpp"
int main(int argc, char **argv) {
    // read the reference's H2O MO file (24 x 5 doubles), write it back at offset 0
    bsgpu::Matrix<double> mo(24, 5);
    mo.read_from_file(argv[1]);
    mo.write_to_file(argv[2]);
    // a size_t matrix with an element offset: the keys file from its 10th entry
    bsgpu::Matrix<size_t> k(4, 1);
    k.read_from_file(argv[3], 10);
    printf("%.17g %zu %zu\n", mo(3, 2), k(0, 0), k(3, 0));
    bsgpu::Matrix<double> big(1000, 1000);
    big.read_from_file(argv[1]);  // too small: exits 1 with a message
    return 0;
}
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("facade")
    src = d / "io.cpp"
    src.write_text(PROG)
    exe = d / "io"
    subprocess.check_call([gxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    return exe, d


def test_matrix_file_format_matches_reference(prog):
    exe, d = prog
    mo_file = os.path.join(GOLDEN, "h2o_occ_mo.bin")
    key_file = os.path.join(GOLDEN, "h2o_v2m_key.bin")
    out = d / "mo_out.bin"
    r = subprocess.run([str(exe), mo_file, str(out), key_file], capture_output=True, text=True)
    assert r.returncode == 1 and "too small" in r.stderr  # the oversized read is refused like the reference's assert
    ref = np.fromfile(mo_file)[:120]
    assert out.read_bytes() == ref.tobytes()  # byte-identical round trip
    mo = ref.reshape(5, 24).T  # column-major 24 x 5
    keys = np.fromfile(key_file, dtype=np.uint64)
    v, k0, k3 = r.stdout.split()
    assert float(v) == mo[3, 2] and int(k0) == keys[10] and int(k3) == keys[13]


@pytest.mark.parametrize("name", ["occ_ri_k_step", "3c_2c_transform", "strassen"])
def test_drivers_print_usage(name):
    exe = os.path.join(ROOT, "strassen_gb300", "drivers", "bin", name)
    if not os.path.exists(exe):
        pytest.skip("drivers not built (strassen_gb300.build.build_drivers)")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith("Usage:")
