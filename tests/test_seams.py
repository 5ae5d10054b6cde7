"""The reference-side binding compiles against the reference's own headers.

tests/integration/seams.cpp holds the bodies a maintainer of the reference
puts in place of its four inner seams (calinternalForce_CSRformat,
timeIntegration_LM, cluster_PARDISO_64Solver, pdfemAssembleEquasSys_CSRformat)
and of its FC 1 crack-growth step (b_cracPropag_qusiaStatic_BYKeq).
Compiling it with the reference's HeaderFiles/Solver, the MPI/MKL shim headers
and include/pdx.h checks that the ABI's prototypes take the reference's
argument types (long long CSR indices, Vector::cdp_vecCoeff) without casts.
"""
import os
import shutil
import subprocess

import pytest

from conftest import REPO, reference_tree

SEAMS = os.path.join(REPO, "tests", "integration", "seams.cpp")


def _compile(include_dir: str):
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present (set PDX_REFERENCE)")
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    cmd = [cxx, "-fsyntax-only", "-std=c++17", "-include", "memory", "-DMKL_ILP64", "-w",
           "-I" + os.path.join(REPO, "oracle", "ref", "shim"), "-I" + os.path.join(ref, "HeaderFiles", "Solver"),
           "-I" + include_dir, SEAMS]
    return subprocess.run(cmd, capture_output=True, text=True)


def test_seams_compile_against_reference_headers():
    r = _compile(os.path.join(REPO, "include"))
    assert r.returncode == 0, r.stderr


def test_seam_types_are_checked(tmp_path):
    """An int64_t* prototype (long on LP64) is what the reference's long long*
    cannot bind to: the same compile must then fail, or the test above would
    check nothing."""
    src = open(os.path.join(REPO, "include", "pdx.h")).read()
    bad = src.replace("long long n, const long long* ia, const long long* ja",
                      "int64_t n, const int64_t* ia, const int64_t* ja")
    assert bad != src
    (tmp_path / "pdx.h").write_text(bad)
    r = _compile(str(tmp_path))
    assert r.returncode != 0 and "long long" in r.stderr
