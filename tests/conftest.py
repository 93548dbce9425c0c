import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _have_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def api():
    from strassen_gb300 import build

    build.build()
    from strassen_gb300 import api as A

    return A


@pytest.fixture(scope="session")
def ctx(api):
    return api.Context(0)


@pytest.fixture(scope="session")
def h2o():
    n_bf, n_aux, n_occ, n_vec2 = 24, 113, 5, 322
    ints = np.fromfile(os.path.join(GOLDEN, "h2o_3c_ints_PQm12.bin")).reshape(n_aux, n_vec2).T.copy(order="F")
    x3c = np.fromfile(os.path.join(GOLDEN, "h2o_3c_ints.bin")).reshape(n_aux, n_vec2).T.copy(order="F")
    v = np.fromfile(os.path.join(GOLDEN, "h2o_2c_inv05.bin")).reshape(n_aux, n_aux).T.copy(order="F")
    c = np.fromfile(os.path.join(GOLDEN, "h2o_occ_mo.bin")).reshape(n_occ, n_bf).T.copy(order="F")
    keys = np.fromfile(os.path.join(GOLDEN, "h2o_v2m_key.bin"), dtype=np.uint64)
    gold = np.load(os.path.join(GOLDEN, "h2o_golden.npz"))
    return dict(n_bf=n_bf, n_aux=n_aux, n_occ=n_occ, n_vec2=n_vec2, ints=ints, x3c=x3c, v=v, c=c, keys=keys,
                gold=gold)


@pytest.fixture(scope="session")
def ref_cases():
    return np.load(os.path.join(GOLDEN, "ref_cases.npz"))


def same_bits(a, b):
    """bit-identical up to the sign of zero"""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))
