"""FC 1: SIFs from the interaction integral, crack growth, PD-region growth
and the load-ratio control of the quasi-static loop, against the reference
itself (tests/golden/pe31_fc1*.npz, made by make_golden.py's fc1_cases from
the reference's own b_cracPropag_qusiaStatic_BYKeq run through its
quasi-static loop).

Two 31 x 31-node FE plates with an edge pre-crack, 24 increments each:
pe31_fc1 plane stress with the default path radius and growth step;
pe31_fc1m plane strain with FC 1 4 1.5 and me = 1.5 (growth also makes the
FE elements next to the new crack elements PD).  The crack first grows at
increment 19 (pe31_fc1) or 18 (pe31_fc1m) and then at every increment, with
the load held."""
import numpy as np
import pytest

from conftest import case_cmd, golden, rel

import pdx

CASES = ["pe31_fc1", "pe31_fc1m"]


def _moves(g):
    """Per increment the tips after the FC 1 pass and which cracks moved."""
    tips = g["crack_rows"][:, :, 1:3]
    prev = np.concatenate([tips[:1], tips[:-1]])
    return tips, np.any(tips != prev, axis=2)


def test_fc1_goldens_grow_the_crack_and_the_pd_region():
    for name in CASES:
        g = golden(name)
        tips, moved = _moves(g)
        region = g["region_rows"]
        n_moves = int(moved.sum())
        assert n_moves >= 5
        # a moved tip holds the load (addLoad false) and grows the PD region
        np.testing.assert_array_equal(region[:, 2] == 0, moved.any(axis=1))
        assert region[-1, 0] > region[0, 0] and region[-1, 1] > region[0, 1]
        # the tip moves by dcf * min_delta along the kink angle, mostly along +x
        step = np.linalg.norm(np.diff(tips[:, 0], axis=0), axis=1)
        assert np.all((step == 0) | (np.abs(step - step.max()) < 1e-12))
        assert tips[-1, 0, 0] > tips[0, 0, 0]


@pytest.mark.parametrize("name", CASES)
def test_crack_advance_reproduces_the_reference_region_growth(built, name):
    """The reference's tip sequence replayed through pdx_crack_advance on a
    host-only model: PD elements (in the reference's civ_pdeIDX order),
    families (appended in its order), members and bond states after the
    last growth are identical."""
    g = golden(name)
    tips, moved = _moves(g)
    m = pdx.Model(case_cmd("pe31", name), device=-1)
    n_fam0 = m.array_len("fam_off") - 1
    for i in range(tips.shape[0]):
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
            assert m.array_len("pde_idx") == int(g["region_rows"][i, 0])
            assert m.array_len("fam_off") - 1 == int(g["region_rows"][i, 1])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
    np.testing.assert_array_equal(m.array("fam_members"), g["fam_members_final"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state_final"])
    assert m.array_len("fam_off") - 1 > n_fam0
    cs = m.crack_state()
    np.testing.assert_array_equal(cs[:, 2:4], tips[-1])


def _pattern_from_definition(m):
    """CSR pattern and scatter-map offsets from their definition: node k's
    rows hold its family members and the nodes of the FE elements around it;
    the offset of neighbour n counts the active DOFs of the row's nodes
    below n."""
    D = m.dim
    eq = m.array("eq").reshape(-1, D)
    N = eq.shape[0]
    off, mem = m.array("fam_off"), m.array("fam_members")
    conn, nn = m.array("conn").reshape(-1, 8), m.array("elem_nn")
    rows = [set() for _ in range(N)]
    for f in range(len(off) - 1):
        rows[mem[off[f]]].update(mem[off[f]:off[f + 1]].tolist())
    for e in m.array("fe_idx"):
        el = conn[e, :nn[e]].tolist()
        for a in el:
            rows[a].update(el)
    ia, ja = [0], []
    for k in range(N):
        cols = [c for j in sorted(rows[k]) for c in eq[j] if c >= 0]
        for d in range(D):
            if eq[k, d] >= 0:
                ja.extend(cols)
                ia.append(len(ja))
    return np.array(ia), np.array(ja), rows, (eq >= 0).sum(axis=1)


@pytest.mark.parametrize("name", CASES)
def test_grown_model_keeps_pattern_and_scatter_map_consistent(built, name):
    """After the reference's growth sequence, the CSR pattern (only the rows
    of the new PD elements' nodes are rebuilt) and the assembly's scatter map
    equal their definitions."""
    g = golden(name)
    tips, moved = _moves(g)
    m = pdx.Model(case_cmd("pe31", name), device=-1)
    for i in range(tips.shape[0]):
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
    ia, ja, rows, nact = _pattern_from_definition(m)
    np.testing.assert_array_equal(m.array("csr_ia"), ia)
    np.testing.assert_array_equal(m.array("csr_ja"), ja)
    off, mem, rel_bond = m.array("fam_off"), m.array("fam_members"), m.array("rel_bond")
    b = 0
    for f in range(len(off) - 1):
        k = mem[off[f]]
        for q in range(off[f] + 1, off[f + 1]):
            if nact[k]:
                assert rel_bond[b] == sum(nact[j] for j in rows[k] if j < mem[q])
            b += 1


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_fc1_quasi_static_run_matches_reference(built, name):
    """All 24 increments through pdx_quasi_step: per increment the tips
    (to 1e-9 of the plate), KI and KII (1e-6 of the largest |K|), Keq
    against K_Ic (the same growth decisions), the PD-region size and the
    free displacements (1e-8); after the last increment the PD elements,
    families, members and bond states exactly, and the reaction forces."""
    g = golden(name)
    rows, region = g["crack_rows"], g["region_rows"]
    with pdx.Model(case_cmd("pe31", name), device=0, precision=0) as m:
        free = m.array("eq") >= 0
        kmax = np.abs(rows[:, :, 3:5]).max()
        worst_u = worst_k = 0.0
        m.quasi_init()
        for i in range(rows.shape[0]):
            info = m.quasi_step(2)
            assert info.converged
            cs = m.crack_state()
            # a tip moves along the kink angle from KII/KI: 1e-9 of the plate
            assert np.abs(cs[:, 2:4] - rows[i, :, 1:3]).max() <= 1e-9 * 0.03, f"increment {i + 1}"
            worst_k = max(worst_k, float(np.abs(cs[:, 4:6] - rows[i, :, 3:5]).max()) / kmax)
            np.testing.assert_array_equal(cs[:, 7] == 1, region[i, 2] == 0)
            assert m.array_len("pde_idx") == int(region[i, 0])
            assert m.array_len("fam_off") - 1 == int(region[i, 1])
            u, _, _, bs = m.state()
            worst_u = max(worst_u, rel(u.reshape(-1)[free], g["u_traj"][i].reshape(-1)[free]))
        rf = m.reaction_forces()
        np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
        np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
        np.testing.assert_array_equal(m.array("fam_members"), g["fam_members_final"])
        np.testing.assert_array_equal(bs, g["bond_state_final"])
    print(f"\n[{name}] worst free-displacement error {worst_u:.2e}, worst K error {worst_k:.2e} of max |K|, "
          f"{int(g['region_rows'][-1, 0])} PD elements, {int((bs == 0).sum())} broken bonds")
    assert worst_u < 1e-8
    assert worst_k < 1e-6
    ref_rf = g["rf_rows"]
    assert rf.shape[0] == ref_rf.shape[0] + 1
    assert np.abs(rf[1:, 1:4] - ref_rf[:, 2:5]).max() <= 1e-7 * np.abs(ref_rf[:, 2:5]).max()


@pytest.mark.gpu
def test_fc1_run_writes_the_crack_path_file(built, tmp_path):
    """pdx_run on an FC 1 deck writes <title>_cp.out with the reference's
    header and one row per increment (scientific, 4 digits)."""
    with pdx.Model(case_cmd("pe31", "pe31_fc1"), device=0, precision=0) as m:
        m.run(str(tmp_path))
    lines = open(tmp_path / "pe31_cp.out").read().splitlines()
    assert lines[0] == "crack ID\t tip_x\t tip_y \t KI \tKII \t Keq"
    assert len(lines) == 1 + 24
    g = golden("pe31_fc1")
    last = lines[-1].split("\t")
    assert float(last[1]) == pytest.approx(g["crack_rows"][-1, 0, 1], rel=1e-3)
    assert float(last[3]) == pytest.approx(g["crack_rows"][-1, 0, 3], rel=1e-3)


def _bench_plate(tmp_path):
    """The 201 x 201-node FC 1 bench plate, regenerated and checked against
    the digest of the inputs the reference ran."""
    import hashlib
    import meshgen
    mesh, kw = meshgen.fc1_bench_case()
    cmd = meshgen.write_case(mesh, str(tmp_path), "pe201_fc1", **kw)
    h = hashlib.sha256()
    for ext in (".in", ".lis"):
        h.update(open(str(tmp_path / ("pe201_fc1" + ext)), "rb").read())
    g = golden("pe201_fc1")
    assert h.hexdigest() == str(g["input_sha256"])
    return cmd, g


def test_crack_advance_reproduces_the_reference_region_growth_on_the_bench_plate(built, tmp_path):
    cmd, g = _bench_plate(tmp_path)
    tips, moved = _moves(g)
    m = pdx.Model(cmd, device=-1)
    for i in range(tips.shape[0]):
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
    np.testing.assert_array_equal(m.array("fam_members"), g["fam_members_final"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state_final"])


@pytest.mark.gpu
@pytest.mark.parametrize("method", [2, 8])
def test_fc1_bench_plate_matches_reference(built, tmp_path, method):
    """The 201 x 201-node bench plate (80,199 equations), 15 increments with
    BiCGStab (method 2) and with the two-level BiCGStab (method 8, whose
    coarse inverse is re-formed after each growth): the reference's ten
    growth steps and its arrest at increment 14, tips to 1e-9 of the plate,
    KI and KII to 1e-6 of the largest |K|, and the final PD elements,
    families and bonds exactly."""
    cmd, g = _bench_plate(tmp_path)
    rows, region = g["crack_rows"], g["region_rows"]
    kmax = np.abs(rows[:, :, 3:5]).max()
    worst_k = 0.0
    with pdx.Model(cmd, device=0, precision=0) as m:
        m.quasi_init()
        for i in range(rows.shape[0]):
            assert m.quasi_step(method).converged
            cs = m.crack_state()
            assert np.abs(cs[:, 2:4] - rows[i, :, 1:3]).max() <= 1e-9 * 0.03, f"increment {i + 1}"
            worst_k = max(worst_k, float(np.abs(cs[:, 4:6] - rows[i, :, 3:5]).max()) / kmax)
            np.testing.assert_array_equal(cs[:, 7] == 1, region[i, 2] == 0)
        _, _, _, bs = m.state()
        np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
        np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
        np.testing.assert_array_equal(bs, g["bond_state_final"])
        rf = m.reaction_forces()
    print(f"\n[pe201_fc1, method {method}] worst K error {worst_k:.2e} of max |K|")
    assert worst_k < 1e-6
    ref_rf = g["rf_rows"]
    assert np.abs(rf[1:, 1:4] - ref_rf[:, 2:5]).max() <= 1e-6 * np.abs(ref_rf[:, 2:5]).max()


EXAMPLES = [("DCT", "DCT_quasiStatic_FC1"), ("DiagPlate", "DiagPlate_quasistatic_FC1"),
            ("plateCrack", "platCrack_quasiStatic_FC1")]


@pytest.mark.parametrize("folder,name", EXAMPLES)
def test_crack_advance_on_the_reference_example_decks(built, folder, name):
    """The reference's own FC 1 example decks (read in the reference tree;
    skipped without it): their crack paths, as the reference's loop produced
    them (tests/golden/ex_*_fc1.npz), replayed through pdx_crack_advance give
    the reference's PD elements, families, members and bond states: a disk
    meshed with triangles and quadrilaterals (DCT, one crack), and two cracks
    growing from a plate's centre in opposite directions (DiagPlate, 48
    growth increments of 54; plateCrack), inside a PD region laid out along
    the crack path in advance."""
    import hashlib
    import os
    from conftest import reference_tree
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    g = golden("ex_" + folder + "_fc1")
    src = os.path.join(ref, "examples", folder)
    cmd = os.path.join(src, name + ".in")
    lis = [ln.split()[1] for ln in open(cmd) if ln.startswith("MSHFILE")][0]
    h = hashlib.sha256()
    for f in (cmd, os.path.join(src, lis)):
        h.update(open(f, "rb").read())
    assert h.hexdigest() == str(g["input_sha256"])
    tips, moved = _moves(g)
    m = pdx.Model(cmd, device=-1)
    for i in range(tips.shape[0]):
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
            assert m.array_len("pde_idx") == int(g["region_rows"][i, 0])
    np.testing.assert_array_equal(m.array("pde_idx"), g["pde_final"])
    np.testing.assert_array_equal(m.array("fam_off"), g["fam_off_final"])
    np.testing.assert_array_equal(m.array("fam_members"), g["fam_members_final"])
    np.testing.assert_array_equal(m.array("bond_state0"), g["bond_state_final"])
    print(f"\n[{folder}] {int(moved.any(axis=1).sum())} growth increments, {m.array_len('pde_idx')} PD elements, "
          f"{int((m.array('bond_state0') == 0).sum())} broken bonds")


@pytest.mark.gpu
def test_static_solve_reports_the_sifs_of_the_quasi_static_increment(built, tmp_path):
    """A static solve with FC 1 evaluates the cracks once (the static
    solver's failure pass): with the top edge held at 2e-7 m it is the second
    increment of pe31_fc1 (the first carries no load), so KI, KII and Keq
    equal the reference's for that increment, and the tip does not move."""
    import meshgen
    m0 = meshgen.plate_edge_crack(n=31, KIc=1.0e6, title="pe31")
    m0.ebcs[2].value = 2e-7
    m0.ebcs[2].velocity = None
    cmd = meshgen.write_case(m0, str(tmp_path), "pe31_static", solver="STATIC", dt=1.0, nsteps=1, save=1,
                             factor=3.015, nlf=1.0, lumped=False, fc="1", extra=["SOLVE BICGSTAB 1e-13 20000"])
    g = golden("pe31_fc1")
    with pdx.Model(cmd, device=0, precision=0) as m:
        m.run(str(tmp_path / "out"))
        cs = m.crack_state()
    ref = g["crack_rows"][1, 0]
    assert cs[0, 7] == 0
    np.testing.assert_allclose(cs[0, 2:4], ref[1:3], rtol=0, atol=1e-15)
    np.testing.assert_allclose(cs[0, 4:7], ref[3:6], rtol=1e-7)


@pytest.mark.parametrize("name", CASES)
def test_fc1_oracle_reproduces_the_reference_sifs(built, name):
    """The CPU restatement (oracle/fc1_oracle.py) pinned against the
    reference: on the reference's own displacements of every increment, with
    the set-up grown as the reference grew it, it gives the reference's KI
    and KII (1e-9 of the largest |K|), its growth decisions and its new tips."""
    import orc
    from fc1_oracle import Fc1Oracle
    g = golden(name)
    rows = g["crack_rows"]
    tips, moved = _moves(g)
    mr, dcf = (4.0, 1.5) if name == "pe31_fc1m" else (6.0, 1.0)
    m = pdx.Model(case_cmd("pe31", name), device=-1)
    kmax = np.abs(rows[:, :, 3:5]).max()
    worst = 0.0
    ev = None
    for i in range(rows.shape[0]):
        if ev is None:
            ev = Fc1Oracle(m, orc.Oracle(m), mr=mr, dcf=dcf)
        cs = m.crack_state()[0]
        KI, KII, _, keq, new_tip = ev.evaluate([cs[0:2], cs[2:4]], g["u_traj"][i], m.array("bond_state0"))
        worst = max(worst, abs(KI - rows[i, 0, 3]) / kmax, abs(KII - rows[i, 0, 4]) / kmax)
        assert (new_tip is not None) == bool(moved[i, 0]), f"increment {i + 1}"
        if moved[i].any():
            np.testing.assert_allclose(new_tip, tips[i, 0], rtol=0, atol=1e-12)
            m.crack_advance(tips[i], moved[i])
            ev = None
    print(f"\n[{name}] oracle vs reference: worst K difference {worst:.2e} of max |K|")
    assert worst < 1e-9


@pytest.mark.parametrize("folder,name", EXAMPLES)
def test_fc1_oracle_on_the_reference_example_decks(built, folder, name):
    """The FC 1 restatement on the reference's own example decks (read in the
    reference tree; skipped without it), at the first growth increment and
    the last, on the reference's displacements and with the set-up grown as
    the reference grew it: every crack's growth decision and new tip, and
    the KI and KII the reference writes (its last crack's)."""
    import os
    import orc
    from conftest import reference_tree
    from fc1_oracle import Fc1Oracle
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    g = golden("ex_" + folder + "_fc1")
    cmd = os.path.join(ref, "examples", folder, name + ".in")
    fc = [ln.split() for ln in open(cmd) if ln.split()[:2] == ["FC", "1"]][0]
    mr, dcf = (float(fc[2]), float(fc[3])) if len(fc) > 3 else (6.0, 1.0)
    rows = g["crack_rows"]
    tips, moved = _moves(g)
    kmax = np.abs(rows[:, :, 3:5]).max()
    m = pdx.Model(cmd, device=-1)
    checked = 0
    for i in range(rows.shape[0]):
        if i in set(g["u_sel_inc"].tolist()):
            u = g["u_sel"][list(g["u_sel_inc"]).index(i)]
            ev = Fc1Oracle(m, orc.Oracle(m), mr=mr, dcf=dcf)
            cs = m.crack_state()
            res = [ev.evaluate([c[0:2], c[2:4]], u, m.array("bond_state0")) for c in cs]
            for ck, (_, _, _, _, new_tip) in enumerate(res):
                assert (new_tip is not None) == bool(moved[i, ck]), f"increment {i + 1}, crack {ck}"
                if new_tip is not None:
                    np.testing.assert_allclose(new_tip, tips[i, ck], rtol=0, atol=1e-12)
            KI, KII = res[-1][0], res[-1][1]
            assert abs(KI - rows[i, 0, 3]) <= 1e-9 * kmax and abs(KII - rows[i, 0, 4]) <= 1e-9 * kmax
            checked += 1
        if moved[i].any():
            m.crack_advance(tips[i], moved[i])
    assert checked == len(g["u_sel_inc"])


def test_crack_api_edge_cases(built, tmp_path):
    """pdx_crack_state / pdx_crack_advance on host-only models: the
    pre-cracks as read, no growth without a moved crack, a 2D model without
    cracks, and a 3D model refused."""
    import meshgen
    m = pdx.Model(case_cmd("pe31", "pe31_fc1"), device=-1)
    cs = m.crack_state()
    assert cs.shape == (1, 8)
    np.testing.assert_allclose(cs[0, :4], [0.25e-3, 0.0155, 0.41 * 0.03, 0.0155], rtol=1e-12)
    assert np.all(cs[0, 4:] == 0)
    before = m.array("pde_idx").copy()
    m.crack_advance(np.array([[0.02, 0.0155]]), np.array([0], dtype=np.uint8))
    np.testing.assert_array_equal(m.array("pde_idx"), before)
    np.testing.assert_array_equal(m.crack_state(), cs)
    plain = meshgen.plate2d(11, 11, 1e-3, pd_mask=lambda c: c[:, 0] < 0.005, title="nc")
    cmd = meshgen.write_case(plain, str(tmp_path), "nc", solver="QUASI-STATIC", dt=1.0, nsteps=2, save=2,
                             factor=3.015, nlf=1.0, lumped=False, fc="1")
    assert pdx.Model(cmd, device=-1).crack_state().shape == (0, 8)
    box = pdx.Model(case_cmd("b13", "b13_explicit"), device=-1)
    with pytest.raises(pdx.PdxError) as e:
        box.crack_advance(np.zeros((1, 2)), np.ones(1, dtype=np.uint8))
    assert e.value.code == 3


@pytest.mark.parametrize("folder,name", EXAMPLES)
def test_example_deck_setups_match_reference(built, folder, name):
    """The library's host set-up and the oracle's own (orc_setup) of the
    reference's FC 1 example decks (read in the reference tree; skipped
    without it) against the reference's set-up, as SHA-256 digests of DOFs,
    families, members, bond states and the CSR pattern."""
    import hashlib
    import os
    import orc_setup
    from conftest import reference_tree
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    g = golden("ex_" + folder + "_fc1")
    cmd = os.path.join(ref, "examples", folder, name + ".in")

    def digest(a):
        return hashlib.sha256(np.asarray(a, dtype=np.int64).reshape(-1).astype("<i8").tobytes()).hexdigest()
    names = ("eq", "fam_off", "fam_members", "bond_state0", "csr_ia", "csr_ja")
    lib_model = pdx.Model(cmd, device=-1)
    oracle_model = orc_setup.load(cmd, pattern=True)
    for n in names:
        ref_digest = str(g["setup_" + n + "_sha256"])
        assert digest(lib_model.array(n)) == ref_digest, ("library", n)
        assert digest(oracle_model.array(n)) == ref_digest, ("oracle", n)
