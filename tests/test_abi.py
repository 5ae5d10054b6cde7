"""The C-ABI library loads and exports every entry point include/pdx.h declares
(no compute: CPU only)."""
import ctypes
import os
import re

from conftest import REPO

import pdx


def declared_symbols():
    src = open(os.path.join(REPO, "include", "pdx.h")).read()
    return sorted(set(re.findall(r"\b(pdx_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_seams():
    names = declared_symbols()
    for n in ("pdx_model_create_from_cmd", "pdx_internal_force", "pdx_explicit_step_host", "pdx_assemble_csr",
              "pdx_solve_csr", "pdx_run"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(pdx.EXPORTED) <= set(declared_symbols())


def test_version_and_error_string(built):
    lib = pdx.lib()
    assert lib.pdx_version().startswith(b"pdlsm")
    assert isinstance(lib.pdx_last_error(), bytes)
