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
