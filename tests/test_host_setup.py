"""Host setup (parsers + pdsolve::setDatModel restatement) against the
reference's own setup dumps, and input-format round trips.  CPU only."""
import os
import tempfile

import numpy as np
import pytest

from conftest import case_cmd, golden

import meshgen
import pdx

CASES = [("p21", "p21_explicit"), ("b13", "b13_explicit")]


@pytest.mark.parametrize("case,cmd", CASES)
def test_setup_matches_reference(built, case, cmd):
    g = golden(case + "_setup")
    m = pdx.Model(case_cmd(case, cmd), device=-1)
    np.testing.assert_array_equal(m.array("eq"), g["eq"].reshape(-1))
    np.testing.assert_array_equal(m.array("node_type"), g["node_type"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off"])
    np.testing.assert_array_equal(m.array("fam_members") + 1, g["fam_members"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state0"])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_idx"])
    np.testing.assert_array_equal(m.array("fe_idx"), g["fe_idx"])
    np.testing.assert_array_equal(m.array("csr_ia"), g["csr_ia"])
    np.testing.assert_array_equal(m.array("csr_ja"), g["csr_ja"])
    # volumes, horizons and PD volumes are computed in the reference's operation order
    np.testing.assert_array_equal(m.array("vol_node"), g["vol_node"])
    np.testing.assert_array_equal(m.array("vol_elem"), g["vol_elem"])
    np.testing.assert_array_equal(m.array("fam_horizon"), g["fam_horizon"])
    np.testing.assert_array_equal(m.array("fam_cdv"), g["fam_cdv"])
    np.testing.assert_array_equal(m.array("geom"), g["geom"])
    nn = 2 if m.dim == 2 else 4
    mine = sorted(tuple(r[:nn]) for r in m.array("pdbe").reshape(-1, 4) + 1)
    ref = sorted(tuple(r[:nn]) for r in g["pdbe"])
    assert mine == ref


def test_lumped_mass_matches_reference(built):
    for case, cmd in CASES:
        m = pdx.Model(case_cmd(case, cmd), device=-1)
        np.testing.assert_array_equal(m.array("mass"), golden(case + "_explicit")["mass"])


def test_meshgen_roundtrip(tmp_path, built):
    mesh = meshgen.plate_strip_crack(n=15, L=0.02)
    cmd = meshgen.write_case(mesh, str(tmp_path), "rt", solver="DYNAMIC", dt=1e-8, nsteps=3, save=1,
                             factor=3.015, nlf=1.0, fc="3 1e-3 7 0.05")
    m = pdx.Model(cmd, device=-1)
    assert m.info.n_node == mesh.n_node and m.info.n_elem == mesh.n_elem
    np.testing.assert_array_equal(m.array("X").reshape(-1, 3), mesh.X)
    conn = m.array("conn").reshape(-1, 8)[:, :4] + 1
    np.testing.assert_array_equal(conn, mesh.elems)
    assert m.info.fail_flag == 3 and m.info.s0 == 1e-3 and abs(m.info.s0_pert - 0.05) < 1e-15
    mat = m.array("material")
    assert int(mat[11]) == 7


def test_hole_mesh_has_no_orphans(built, tmp_path):
    mesh = meshgen.box_hole(nx=13, ny=9, nz=3, h=1e-3, radius=2e-3, pd_x=8, pd_y=6)
    used = np.zeros(mesh.n_node, bool)
    used[mesh.elems.ravel() - 1] = True
    assert used.all()
    cmd = meshgen.write_case(mesh, str(tmp_path), "bh", solver="DYNAMIC", dt=1e-8, nsteps=1, save=1,
                             factor=3.015, nlf=1.0)
    m = pdx.Model(cmd, device=-1)
    assert (m.array("vol_node") > 0).all()


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)


def test_errors_are_returned_not_exit(built, tmp_path):
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "missing.in"), device=-1)
    assert e.value.code == 1
    _write(tmp_path / "bad.in", "MSHFILE nothere.lis\nSOLVER DYNAMIC\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "bad.in"), device=-1)
    assert e.value.code == 1
    mesh = meshgen.plate_strip_crack(n=11, L=0.01)
    meshgen.write_lis(mesh, str(tmp_path / "m.lis"))
    _write(tmp_path / "s.in", "MSHFILE m.lis\nSOLVER SIDEWAYS\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "s.in"), device=-1)
    assert e.value.code == 2
    _write(tmp_path / "p.in", "MSHFILE m.lis\nSOLVER DYNAMIC\nPRECISION HALF\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "p.in"), device=-1)
    assert e.value.code == 2
    _write(tmp_path / "f.in", "MSHFILE m.lis\nSOLVER DYNAMIC\nFC 3 -1\n")
    with pytest.raises(pdx.PdxError):
        pdx.Model(str(tmp_path / "f.in"), device=-1)
    _write(tmp_path / "g.in", "MSHFILE m.lis\nSOLVER QUASI-STATIC\nSOLVE GMRES 1e-9 400\n")
    pdx.Model(str(tmp_path / "g.in"), device=-1)
    _write(tmp_path / "h.in", "MSHFILE m.lis\nSOLVER QUASI-STATIC\nSOLVE LU\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "h.in"), device=-1)
    assert e.value.code == 2
    # an unknown Krylov method is refused before any device work
    ia = np.array([0, 1], np.int64)
    with pytest.raises(pdx.PdxError) as e:
        pdx.solve_csr(ia, np.array([0], np.int64), np.array([2.0]), np.array([1.0]), method=5)
    assert e.value.code == 4


def test_bare_fc3_breaks_nothing_as_the_reference(built, tmp_path):
    """The reference reads FC 3 without a value and breaks no bond with it
    (its stretch criterion is never called); such decks still run."""
    mesh = meshgen.plate_strip_crack(n=11, L=0.01)
    meshgen.write_case(mesh, str(tmp_path), "b", solver="DYNAMIC", dt=1e-8, nsteps=2, save=2, factor=3.015, nlf=1.0,
                       fc="3")
    m = pdx.Model(str(tmp_path / "b.in"), device=-1)
    assert m.info.fail_flag == 0


def test_duplicate_dof_and_unsupported_elements(built, tmp_path):
    mesh = meshgen.plate_strip_crack(n=11, L=0.01)
    mesh.ebcs.append(meshgen.EBC(0, 0.0, mesh.ebcs[0].nodes[:2]))
    meshgen.write_lis(mesh, str(tmp_path / "d.lis"))
    _write(tmp_path / "d.in", "MSHFILE d.lis\nSOLVER DYNAMIC\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "d.in"), device=-1)
    assert "repeatly" in str(e.value)
    # a 2D record repeating its third node is a 3-node triangle (read); a 3D
    # record collapsing a face (a tetrahedron or prism) is refused
    tri = meshgen.plate_strip_crack(n=11, L=0.01)
    tri.elems[0, 3] = tri.elems[0, 2]
    meshgen.write_lis(tri, str(tmp_path / "t.lis"))
    _write(tmp_path / "t.in", "MSHFILE t.lis\nSOLVER DYNAMIC\n")
    assert pdx.Model(str(tmp_path / "t.in"), device=-1).array("elem_nn")[0] == 3
    tet = meshgen.box3d(4, 4, 4, 1e-3, pd_mask=lambda c: c[:, 0] < 0)
    tet.elems[0, 3] = tet.elems[0, 2]
    meshgen.write_lis(tet, str(tmp_path / "h.lis"))
    _write(tmp_path / "h.in", "MSHFILE h.lis\nSOLVER DYNAMIC\n")
    with pytest.raises(pdx.PdxError) as e:
        pdx.Model(str(tmp_path / "h.in"), device=-1)
    assert e.value.code == 3


def test_compute_without_device_fails_loudly(built):
    m = pdx.Model(case_cmd("p21", "p21_explicit"), device=-1)
    with pytest.raises(pdx.PdxError) as e:
        m.internal_force(np.zeros((m.info.n_node, 2)))
    assert e.value.code == 8
    with pytest.raises(pdx.PdxError):
        m.explicit_advance(1)


def test_command_keywords(built, tmp_path):
    mesh = meshgen.plate_strip_crack(n=11, L=0.01)
    meshgen.write_lis(mesh, str(tmp_path / "k.lis"))
    _write(tmp_path / "k.in", "# comment\nMSHFILE k.lis\nSOLVER QUASI-STATIC\nSETSOLVING 5e-7 12 3 3.5 0.5 2\n"
           "NEWMARK ON 0.6 0.3\nLUMPMASS ON\nEBC 2 1e-6\nVEBC 2 2e-6\nFC 3 2e-3 9 0.1\nPRECISION MIXED\n"
           "SOLVE BJPCG 1e-9 500\nFOO bar\nVTKFORMAT ASCII\n")
    m = pdx.Model(str(tmp_path / "k.in"), device=-1)
    i = m.info
    assert i.solver == 2 and i.dt == 1.0 and i.nsteps == 12 and i.save_freq == 3
    assert i.newmark == 1 and i.lumped == 1 and i.fail_flag == 3 and i.precision == 1
    u0 = m.array("u0").reshape(-1, 2)
    top = mesh.ebcs[2].nodes - 1
    assert np.all(u0[top, 1] == 1e-6)
    dtv = m.array("dtv").reshape(-1, 3)
    assert np.all(dtv[top, 1] == 1.0 * 2e-6)


def test_c3_plate_matches_the_configuration_sizes():
    """C3: 401x401 nodes, PD band over the middle 30 % of the width, 0.2 W
    pre-crack; about 321.6k equations and 9.6e6 nonzeros."""
    d = tempfile.mkdtemp()
    mesh, kw = meshgen.config_c3(nsteps=2)
    cmd = meshgen.write_case(mesh, d, "c3", **kw)
    m = pdx.Model(cmd, device=-1)
    i = m.info
    assert i.dim == 2 and i.n_node == 401 * 401 and i.solver == 2
    assert 315_000 < i.n_eq < 322_000
    assert 9.4e6 < i.nnz < 9.8e6
    assert i.n_fam > 0 and i.fail_flag == 3


def test_step_at_a_time_entry_points_need_a_device():
    """Quasi-static, Newmark and learned entry points on a host-only model
    return NODEVICE (or INVALID before set-up) instead of computing on the CPU."""
    host = pdx.Model(case_cmd("p21", "p21_quasi"), device=-1)
    for call in (host.quasi_init, lambda: host.quasi_step(1), host.newmark_init, lambda: host.newmark_step(4),
                 lambda: host.learned_setup((4, 4), hidden=8)):
        with pytest.raises(pdx.PdxError) as e:
            call()
        assert e.value.code == 8
    for call in (lambda: host.learned_options(1, 60), host.learned_pairs, lambda: host.learned_train(1)):
        with pytest.raises(pdx.PdxError) as e:
            call()
        assert e.value.code in (4, 8)
    assert host.learned_active() is False
    assert host.learned_samples() == 0


@pytest.mark.parametrize("case,cmd", CASES + [("pe31", "pe31_fc1"), ("t21", "t21_explicit")])
def test_scatter_map_offsets_count_the_columns_of_lower_nodes(built, case, cmd):
    """The assembly's scatter map against its definition: the offset of
    neighbour n in node k's rows is the number of active DOFs of the nodes
    below n among k's row nodes (k's family members and the nodes of the FE
    elements around k, sorted, without repeats)."""
    m = pdx.Model(case_cmd(case, cmd), device=-1)
    D = m.dim
    eq = m.array("eq").reshape(-1, D)
    nact = (eq >= 0).sum(axis=1)
    off, mem = m.array("fam_off"), m.array("fam_members")
    fe_conn = m.array("fe_conn").reshape(-1, 8)
    nen = 4 if D == 2 else 8   # a triangle repeats its third node in the fourth slot
    N = eq.shape[0]
    rows = [set() for _ in range(N)]
    for f in range(len(off) - 1):
        rows[mem[off[f]]].update(mem[off[f]:off[f + 1]].tolist())
    for el in fe_conn:
        for a in el[:nen]:
            rows[a].update(el[:nen].tolist())

    def rel(k, n):
        return int(sum(nact[j] for j in rows[k] if j < n))

    rel_bond, rel_self = m.array("rel_bond"), m.array("rel_self")
    b = 0
    for f in range(len(off) - 1):
        k = mem[off[f]]
        if nact[k]:
            assert rel_self[f] == rel(k, k)
        for q in range(off[f] + 1, off[f + 1]):
            if nact[k]:
                assert rel_bond[b] == rel(k, mem[q])
            b += 1
    ptr, adj, rfe = m.array("fe_adj_ptr"), m.array("fe_adj"), m.array("rel_fe").reshape(-1, 8)
    for k in range(N):
        if not nact[k]:
            continue
        for j in range(ptr[k], ptr[k + 1]):
            el = fe_conn[adj[j] >> 3]
            for a in range(nen):
                assert rfe[j, a] == rel(k, el[a])


def _example_decks():
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ex_setups.npz"))
    return sorted({(k.split("__")[0], k.split("__")[1]) for k in g.files})


@pytest.mark.parametrize("folder,deck", _example_decks())
def test_every_reference_example_deck_sets_up_as_the_reference(built, folder, deck):
    """Every example deck of the reference whose mesh is in its tree (read
    there; skipped without it): the library's host set-up and the oracle's
    own give the reference's DOFs, families, members, bond states and CSR
    pattern (SHA-256 digests, tests/golden/ex_setups.npz)."""
    import hashlib
    import sys
    from conftest import REPO, reference_tree
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import orc_setup
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    g = golden("ex_setups")
    cmd = os.path.join(ref, "examples", folder, deck + ".in")

    def digest(a):
        return hashlib.sha256(np.asarray(a, dtype=np.int64).reshape(-1).astype("<i8").tobytes()).hexdigest()
    lib_model = pdx.Model(cmd, device=-1)
    oracle_model = orc_setup.load(cmd, pattern=True)
    for n in ("eq", "fam_off", "fam_members", "bond_state0", "csr_ia", "csr_ja"):
        want = str(g[f"{folder}__{deck}__{n}_sha256"])
        assert digest(lib_model.array(n)) == want, ("library", n)
        assert digest(oracle_model.array(n)) == want, ("oracle", n)
