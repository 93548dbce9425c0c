"""The C ABI library loads and exports every symbol include/bsgpu.h declares
(CPU only: no compute calls)."""
import ctypes
import os
import re

from tests.conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "bsgpu.h")).read()
    # function declarations: a return type at the start of a line, then the name
    decl = r"^\s*(?:bsg_status|int|const\s+char\s*\*)\s*(bsg_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("bsg_matmult", "bsg_matmult_strassen_sparse", "bsg_rik_occ_step", "bsg_rik_kmn_step",
                 "bsg_3c2c_transform",
                 "bsg_bsm_create", "bsg_pool_create", "bsg_tensormult_contract", "bsg_strassen_dryrun"):
        assert must in syms


def test_library_exports_every_declared_symbol(api):
    lib = ctypes.CDLL(os.path.join(ROOT, "strassen_gb300", "libbsgpu.so"))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_string(api):
    assert api.lib.bsg_version() >= 10000
    assert isinstance(api.lib.bsg_last_error(), bytes)


def test_null_arguments_are_rejected(api):
    """argument checks return a status before any device work"""
    assert api.lib.bsg_ctx_create(0, None, None) != 0
    assert api.lib.bsg_bsm_create(None, 4, 4, 2, 2, 0.0, None, None) != 0
    assert b"NULL" in api.lib.bsg_last_error()
    assert api.lib.bsg_matmult(None, None, 0, None, 0, 0.0, 1.0, 0.0, None) != 0
    assert api.lib.bsg_rik_occ_step(None, None, None, 0, None) != 0
    assert api.lib.bsg_rik_kmn_step(None, None, None, None, 0, None) != 0
