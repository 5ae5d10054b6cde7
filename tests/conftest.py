import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "pdlsm-fem_mpi_gb300")
for p in (PKG, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def reference_tree():
    """The reference checkout: PDX_REFERENCE, else the one __graft_entry__.build()
    recorded when it built the oracle's reference build; None when neither exists
    (the GPU machine has no copy)."""
    ref = os.environ.get("PDX_REFERENCE")
    rec = os.path.join(REPO, "oracle", "_ref", "reference_path.txt")
    if not ref and os.path.exists(rec):
        ref = open(rec).read().strip()
    if ref and os.path.isdir(os.path.join(ref, "HeaderFiles", "Solver")):
        return ref
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def built():
    """The library, CLI and oracle, built in-tree if missing."""
    import build as pkg_build
    import orc
    lib = os.path.join(PKG, "lib", "libpdx.so")
    if not os.path.exists(lib):
        pkg_build.build()
    orc.build()
    return lib


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def case_cmd(case: str, name: str) -> str:
    return os.path.join(GOLDEN, "cases", case, name + ".in")


def rel(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
