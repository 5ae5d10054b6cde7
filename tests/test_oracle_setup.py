"""The oracle's own host set-up (oracle/orc_setup.py: readers and
setDatModel restated in numpy, no product code) against the reference's
set-up dumps, bit for bit, at fixture size and, through SHA-256 digests, at
the C1 and C2 configurations' own sizes.  The bench's CPU legs and smoke()
build the oracle on it."""
import hashlib
import os
import sys

import numpy as np
import pytest

from conftest import REPO, case_cmd, golden

sys.path.insert(0, os.path.join(REPO, "oracle"))
import orc_setup  # noqa: E402

import meshgen  # noqa: E402


@pytest.mark.parametrize("case,cmd", [("p21", "p21_explicit"), ("b13", "b13_explicit"), ("t21", "t21_explicit")])
def test_oracle_setup_matches_reference_dump(case, cmd):
    g = golden(case + "_setup")
    h = orc_setup.load(case_cmd(case, cmd))
    np.testing.assert_array_equal(h.array("eq"), g["eq"].reshape(-1))
    np.testing.assert_array_equal(h.array("node_type"), g["node_type"])
    np.testing.assert_array_equal(h.array("fam_off"), g["fam_off"])
    np.testing.assert_array_equal(h.array("fam_members") + 1, g["fam_members"])
    np.testing.assert_array_equal(h.array("bond_state0"), g["bond_state0"])
    np.testing.assert_array_equal(h.array("pde_idx"), g["pde_idx"])
    np.testing.assert_array_equal(h.array("fe_idx"), g["fe_idx"])
    for name in ("vol_node", "vol_elem", "fam_horizon", "fam_cdv", "geom"):
        np.testing.assert_array_equal(h.array(name), g[name])
    nn = 2 if h.dim == 2 else 4
    assert sorted(tuple(r[:nn]) for r in h.array("pdbe") + 1) == sorted(tuple(r[:nn]) for r in g["pdbe"])


def _digests_equal(h, g):
    out = {}
    for k in g.files:
        if not k.endswith("_sha256") or k.startswith(("csr", "input")):
            continue
        a = np.asarray(h.array(k[:-7]), dtype=np.int64).reshape(-1)
        out[k] = hashlib.sha256(a.astype("<i8").tobytes()).hexdigest() == str(g[k])
    return out


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_oracle_setup_matches_reference_at_configuration_size(tmp_path, name):
    mesh, kw = meshgen.config_c1(nsteps=10) if name == "c1" else meshgen.config_c2(nsteps=10)
    cmd = meshgen.write_case(mesh, str(tmp_path), name, **kw)
    h = orc_setup.load(cmd)
    res = _digests_equal(h, golden("c1_size" if name == "c1" else "c2_setup"))
    assert res and all(res.values()), res


@pytest.mark.parametrize("folder,deck", [("DiagPlate", "DiagPlate_static"), ("plateCrack", "platCrack_Static"),
                                         ("plateHole", "platHole_Static")])
def test_oracle_static_assembly_on_reference_example_decks(folder, deck):
    """The oracle (own set-up, CSR pattern and assembly) on the reference's
    static example decks (read in the reference tree; skipped without it):
    the load vector and the stiffness applied to a seeded vector equal the
    reference's (tests/golden/ex_static.npz)."""
    from conftest import reference_tree
    import orc
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    g = golden("ex_static")
    h = orc_setup.load(os.path.join(ref, "examples", folder, deck + ".in"), pattern=True)
    o = orc.Oracle(h)
    v = h.array("u0").copy()
    v[h.array("eq") >= 0] = 0.0
    ia, ja, a, f = o.assemble(v)
    n = len(ia) - 1
    x = np.random.default_rng(7).standard_normal(n)
    kx = np.array([a[ia[r]:ia[r + 1]] @ x[ja[ia[r]:ia[r + 1]]] for r in range(n)])
    want_f, want_kx = g[f"{folder}__{deck}__F"], g[f"{folder}__{deck}__Kx"]
    assert np.linalg.norm(f - want_f) <= 1e-12 * np.linalg.norm(want_f)
    assert np.linalg.norm(kx - want_kx) <= 1e-12 * np.linalg.norm(want_kx)
