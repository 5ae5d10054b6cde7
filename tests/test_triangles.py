"""3-node triangles (pdfemEleTri3N): read from the .lis record whose fourth
node repeats the third, stored in the 4-node tables with zero fourth rows and
columns, constant-strain stiffness, consistent mass and stress.  Against the
reference's own dumps (tests/golden/t21_*.npz, te31_fc1.npz, made by
make_golden.py's tri_cases): t21 is the 21 x 21 plate with a PD strip and a
pre-crack whose left half is split into triangles; te31 the 31 x 31 FC 1
edge-cracked plate split into triangles everywhere."""
import numpy as np
import pytest

from conftest import case_cmd, golden, rel

import pdx

FP64_TOL = 1e-10


def test_setup_with_triangles_matches_reference(built):
    g = golden("t21_setup")
    m = pdx.Model(case_cmd("t21", "t21_explicit"), device=-1)
    assert int((m.array("elem_nn") == 3).sum()) > 0
    np.testing.assert_array_equal(m.array("eq"), g["eq"].reshape(-1))
    np.testing.assert_array_equal(m.array("node_type"), g["node_type"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off"])
    np.testing.assert_array_equal(m.array("fam_members") + 1, g["fam_members"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state0"])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_idx"])
    np.testing.assert_array_equal(m.array("fe_idx"), g["fe_idx"])
    np.testing.assert_array_equal(m.array("csr_ia"), g["csr_ia"])
    np.testing.assert_array_equal(m.array("csr_ja"), g["csr_ja"])
    np.testing.assert_array_equal(m.array("vol_node"), g["vol_node"])
    np.testing.assert_array_equal(m.array("vol_elem"), g["vol_elem"])
    np.testing.assert_array_equal(m.array("fam_horizon"), g["fam_horizon"])
    np.testing.assert_array_equal(m.array("fam_cdv"), g["fam_cdv"])
    mine = sorted(tuple(r[:2]) for r in m.array("pdbe").reshape(-1, 4) + 1)
    ref = sorted(tuple(r[:2]) for r in g["pdbe"])
    assert mine == ref
    np.testing.assert_array_equal(m.array("mass"), golden("t21_explicit")["mass"])


def test_triangle_fc1_growth_replay_matches_reference(built):
    """The reference's crack path on the triangulated FC 1 plate replayed
    through pdx_crack_advance: PD elements, families, members and bonds."""
    g = golden("te31_fc1")
    tips = g["crack_rows"][:, :, 1:3]
    prev = np.concatenate([tips[:1], tips[:-1]])
    moved = np.any(tips != prev, axis=2)
    m = pdx.Model(case_cmd("t21", "te31_fc1"), device=-1)
    for i in range(tips.shape[0]):
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
    np.testing.assert_array_equal(m.array("fam_members"), g["fam_members_final"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state_final"])


@pytest.mark.gpu
def test_explicit_with_triangles_matches_reference(built):
    """60 explicit FP64 steps with FC 3 on the half-triangulated plate."""
    ge = golden("t21_explicit")
    with pdx.Model(case_cmd("t21", "t21_explicit"), device=0, precision=0) as m:
        m.explicit_init()
        done, worst = 0, 0.0
        for i, s in enumerate(ge["u_traj_steps"]):
            m.explicit_advance(int(s) + 1 - done)
            done = int(s) + 1
            u, sig, phi, bs = m.state()
            worst = max(worst, rel(u, ge["u_traj"][i]))
    print(f"\n[t21] explicit FP64 with triangles: worst u error {worst:.2e}")
    assert worst < FP64_TOL
    np.testing.assert_array_equal(bs, ge["bond_state_final"])
    assert rel(sig, ge["sigma_final"]) < FP64_TOL


@pytest.mark.gpu
def test_static_with_triangles_matches_reference(built):
    gs = golden("t21_static")
    host = pdx.Model(case_cmd("t21", "t21s"), device=-1)
    v = host.array("u0").reshape(-1).copy()
    v[host.array("eq") >= 0] = 0.0
    with pdx.Model(case_cmd("t21", "t21s"), device=0, precision=0) as m:
        ia, ja, a, f = m.assemble(1, v)
    np.testing.assert_array_equal(ia, gs["K_ia"])
    np.testing.assert_array_equal(ja, gs["K_ja"])
    assert rel(a, gs["K_a"]) < 1e-12
    assert rel(f, gs["F"]) < 1e-12


@pytest.mark.gpu
def test_triangle_fc1_quasi_static_run_matches_reference(built):
    g = golden("te31_fc1")
    rows, region = g["crack_rows"], g["region_rows"]
    kmax = np.abs(rows[:, :, 3:5]).max()
    worst_k = worst_u = 0.0
    with pdx.Model(case_cmd("t21", "te31_fc1"), device=0, precision=0) as m:
        free = m.array("eq") >= 0
        m.quasi_init()
        for i in range(rows.shape[0]):
            assert m.quasi_step(2).converged
            cs = m.crack_state()
            assert np.abs(cs[:, 2:4] - rows[i, :, 1:3]).max() <= 1e-9 * 0.03, f"increment {i + 1}"
            worst_k = max(worst_k, float(np.abs(cs[:, 4:6] - rows[i, :, 3:5]).max()) / kmax)
            np.testing.assert_array_equal(cs[:, 7] == 1, region[i, 2] == 0)
            u = m.state()[0]
            worst_u = max(worst_u, rel(u.reshape(-1)[free], g["u_traj"][i].reshape(-1)[free]))
        _, _, _, bs = m.state()
        np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
        np.testing.assert_array_equal(bs, g["bond_state_final"])
        rf = m.reaction_forces()
    print(f"\n[te31_fc1] worst K error {worst_k:.2e} of max |K|, worst free-displacement error {worst_u:.2e}")
    assert worst_k < 1e-6 and worst_u < 1e-8
    ref_rf = g["rf_rows"]
    assert np.abs(rf[1:, 1:4] - ref_rf[:, 2:5]).max() <= 1e-7 * np.abs(ref_rf[:, 2:5]).max()
